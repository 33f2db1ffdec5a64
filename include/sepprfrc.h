/*
 * sepprfrc.h - non-bonded pair forces (reference include/sepprfrc.h:49-71).
 */
#ifndef SEP_GB300_SEPPRFRC_H
#define SEP_GB300_SEPPRFRC_H

#include <stdlib.h>
#include <string.h>
#include "sepdef.h"
#include "sepstrct.h"
#include "sepmisc.h"

/*
 * Pair force between the two types in `types` with the potential `fun`
 * cut at `cf` (cf may not exceed sys->cf).  The neighbour list is rebuilt
 * first when sys->neighb_flag is set, honouring the exclusion option.
 * ret->epot is ASSIGNED the pair energy and ret->pot_P accumulates the
 * virial, as in the reference (reference :49-51, source/sepprfrc.c:94-274).
 */
int sep_force_pairs(seppart *ptr, const char *types, double cf,
		    double (*fun)(double, char), sepsys *sys,
		    sepret *retval, const unsigned opt);

/*
 * Lennard-Jones pair force with param = {cut-off, epsilon, sigma, aw}
 * (the order the reference code reads, source/sepprfrc.c:785); the energy
 * is shifted to zero at the cut-off and ADDED to ret->epot
 * (reference :62-64, source/sepprfrc.c:743-1000).
 */
void sep_force_lj(seppart *ptr, const char *types, const double *param,
		  sepsys *sys, sepret *retval, const unsigned opt);

/* Exclusion predicates on the per-particle partner arrays
 * (reference :120-123, source/sepprfrc.c:703-740). */
unsigned int sep_bond_share(seppart *ptr, int j1, int j2);
unsigned int sep_angle_share(seppart *ptr, int j1, int j2);
unsigned int sep_dihed_share(seppart *ptr, int j1, int j2);
unsigned int sep_bonded(seppart *ptr, int i, int j);

#endif
