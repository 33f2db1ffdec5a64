/*
 * sepinit.h - allocation and set-up of particles and the system
 * (reference include/sepinit.h:29-90).
 */
#ifndef SEP_GB300_SEPINIT_H
#define SEP_GB300_SEPINIT_H

#include <stdio.h>
#include "sepdef.h"
#include "sepstrct.h"
#include "sepmisc.h"
#include "sepmol.h"

/* Allocates npart particles with the default type 'A', mass 1 and
 * molindex -1.  nneighb is accepted for compatibility; neighbour lists are
 * kept on the GPU and sized there (reference :29). */
seppart *sep_init(size_t npart, size_t nneighb);

/* Frees the particles and their device state (reference :36). */
void sep_close(seppart *ptr, size_t npart);

/* Allocates and reads particles from an xyz file: the count, the three box
 * lengths, then "type x y z vx vy vz m z" per line (reference :48). */
seppart *sep_init_xyz(double *lbox, int *npart, const char *file, char verbose);

/* Simple-cubic lattice offset by 1.0 (reference :56). */
void sep_set_lattice(seppart *ptr, sepsys sys);

/* Random velocities scaled to the temperature, zero momentum (reference :64). */
void sep_set_vel(seppart *ptr, double temp, sepsys sys);

/* Builds the system structure; the cell grid is sized for cut-off + 0.25
 * (reference :78). */
sepsys sep_sys_setup(double lengthx, double lengthy, double lengthz,
		     double maxsyscf, double dt, size_t npart, size_t update);

/* Frees the topology lists held by the system (reference :85). */
void sep_free_sys(sepsys *ptr);

/* Seeded variants (reference :91-93). */
void sep_set_vel_seed(seppart *ptr, double temp, unsigned int seed, sepsys sys);
void sep_set_vel_type(seppart *ptr, char type, double temp, unsigned int seed,
		      sepsys sys);

#endif
