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

/*
 * DPD pair force of Groot and Warren between the types of `types` within cf:
 * with w = 1 - r, conservative aij w, dissipative -gamma w^2 (rhat . vij)
 * on the predicted velocities pv, gamma = sigma^2/(2 T), and random
 * sigma w dt^(-1/2) theta with theta uniform of unit variance, all along
 * rhat.  On the neighbour list the energy sum aij w^2/2 is ASSIGNED to
 * ret->epot; under SEP_BRUTE it is added, with the conservative virial added
 * to pot_P and the three parts to pot_P_conservative, pot_P_random and
 * pot_P_dissipative (reference :89-101, :172-176,
 * source/sepprfrc.c:278-301, :1007-1235).  The random numbers are this
 * library's counter-based streams (sep_gpu_set_seed), not rand().
 */
void sep_force_dpd(seppart *ptr, const char *types, const double cf, const double aij,
		   const double temp_desired, const double sigma, sepsys *sys, sepret *retval,
		   const unsigned opt);
void sep_dpdforce_neighb(seppart *ptr, const char *types, const double cf, const double aij,
			 const double temp_desired, const double sigma, sepsys *sys,
			 sepret *retval, const unsigned opt);
void sep_dpdforce_brute(seppart *ptr, const char *types, const double cf, const double aij,
			const double temp_desired, const double sigma, sepsys *sys,
			sepret *retval);

/* Exclusion predicates on the per-particle partner arrays
 * (reference :120-123, source/sepprfrc.c:703-740). */
unsigned int sep_bond_share(seppart *ptr, int j1, int j2);
unsigned int sep_angle_share(seppart *ptr, int j1, int j2);
unsigned int sep_dihed_share(seppart *ptr, int j1, int j2);
unsigned int sep_bonded(seppart *ptr, int i, int j);

#endif
