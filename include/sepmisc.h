/*
 * sepmisc.h - helper macros, the built-in pair potentials and the small
 * utilities of the sep C API that the MD-step hot path uses.
 *
 * Declarations follow the reference's include/sepmisc.h; each entry names
 * the line of the reference declaration it stands in for.
 */
#ifndef SEP_GB300_SEPMISC_H
#define SEP_GB300_SEPMISC_H

#include <stdio.h>
#include <stdlib.h>
#include <stdarg.h>
#include <string.h>
#include <math.h>
#include <time.h>
#include <float.h>
#include "sepdef.h"
#include "sepstrct.h"

/* Macros programs use (reference include/sepmisc.h:39-95). */
#define SEP_FLUSH fflush(stdout)
#define SEP_TICTOC clock_t time_then
#define SEP_TIC time_then = clock()
#define SEP_TOC ((int)(1000*(clock()-time_then)/CLOCKS_PER_SEC))%1000
#define sep_rand() ( rand()/(RAND_MAX+1.0) )
#define sep_here(x) { printf("%d\n", x); SEP_FLUSH; }
#define sep_Sq(x) ( (x)*(x) )
#define sep_Abs(x) ( (x) > 0.0 ? (x) : -(x) )
/* minimum-image wrap of one component x of a separation in a box of length y */
#define sep_Wrap(x, y) { if ( (x) > 0.5*(y) ) (x) -= (y); else if ( (x) < -0.5*(y) ) (x) += (y); }
/* periodic wrap of one position component into [0, y) */
#define sep_Periodic(x, y) { if ( (x) > (y) ) (x) -= (y); else if ( (x) < 0.0 ) (x) += (y); }

/* Prints "sep-error -> message" and exits with EXIT_FAILURE (reference :101). */
void sep_error(char *str, ...);
/* Prints "sep-warning -> message" and continues (reference :108). */
void sep_warning(char *str, ...);

/*
 * Built-in pair potentials, f(r^2, 'f') = -dU/dr / r and f(r^2, 'u') = U
 * (reference :115-136).  Passing one of these to sep_force_pairs() selects the
 * matching device kernel; any other function is tabulated on the host.
 */
double sep_lj(double r2, char opt);
double sep_lj_shift(double r2, char opt);
double sep_wca(double r2, char opt);
double sep_spring_x0(double r2, char opt);

/* Writes the particles of the listed types as xyz text (reference :164). */
void sep_save_xyz(seppart *ptr, const char *partnames, const char *file,
		  char *mode, sepsys *sys);

/* Zeroes the forces and sys->max_dist2 (reference :245). */
void sep_reset_force(seppart *ptr, sepsys *sys);
/* Zeroes the molecular force matrix (reference :252). */
void sep_reset_force_mol(sepsys *sys);

/* Counts the particles of one type (reference :285). */
int sep_count_type(seppart *ptr, char type, int npart);

/* Marks the system as threaded; the GPU path ignores the thread count (reference :303). */
void sep_set_omp(unsigned nthreads, sepsys *sys);
/* Sets the neighbour-list skin (reference :311). */
void sep_set_skin(sepsys *sys, double value);

/* Sets mass or charge of every particle of a type (reference :320-330). */
void sep_set_charge(seppart *ptr, char type, double z, sepsys sys);
void sep_set_mass(seppart *ptr, char type, double m, sepsys sys);
/*
 * Box changes.  sep_compress_box scales every edge and coordinate by xi
 * (1/xi when the density is above rhoD; nothing within 1e-6 of it);
 * sep_compress_box_dir (density below rhoD) and sep_compress_box_dir_length
 * (edge above length) scale one edge by xi and its coordinates by xi^(1/3);
 * the Berendsen barostat takes xi = 1 - beta dt (Pd - p) from the current
 * pressure and scales L_z (sep_berendsen) or every edge (sep_berendsen_iso)
 * by xi and the same coordinates by xi^(1/3).  The volume and the sub-box
 * grid follow (reference :181-216, :373-401, source/sepmisc.c:892-1084).
 */
void sep_compress_box(sepatom *ptr, double rhoD, double xi, sepsys *sys);
void sep_compress_box_dir(sepatom *ptr, double rhoD, double xi, int dir, sepsys *sys);
void sep_compress_box_dir_length(sepatom *ptr, double length, double xi, int dir, sepsys *sys);
void sep_berendsen(sepatom *ptr, double Pd, double beta, sepret *ret, sepsys *sys);
void sep_berendsen_iso(sepatom *ptr, double Pd, double beta, sepret *ret, sepsys *sys);

/* Molecular Berendsen barostat (reference :216, source/sepmisc.c:948-990):
 * xi = 1 - beta dt (Pd - p_mol) from sep_mol_pressure_tensor; L_z is scaled
 * by xi, each molecule's centre-of-mass z by xi^(1/3) with its atoms keeping
 * their offsets from it (wrapped once into the box), mol[].x[2] likewise. */
void sep_berendsen_mol(sepatom *ptr, sepmol *mol, double Pd, double beta, sepret *ret, sepsys *sys);

/* Sets the Langevin diffusion coefficient of every particle of a type
 * (reference :449, source/sepmisc.c:1162-1170). */
void sep_set_ldiff(seppart *ptr, char type, double ldiff, sepsys sys);

/* Removes the centre-of-mass momentum of one type (reference :338). */
void sep_reset_momentum(seppart *ptr, const char type, sepsys *sys);

/* Rescales the velocities of one type towards the temperature Td with
 * relaxation time tau, then removes that type's momentum (reference :175,
 * source/sepmisc.c:357-391). */
void sep_relax_temp(seppart *ptr, char type, double Td, double tau, sepsys *sys);

/* Tether force f -= fun(r2, 'f') r, r = x0 - x (minimum image), on the
 * particles of one type (reference :262, source/sepmisc.c:645-670); this
 * implementation takes linear tethers, fun(r2, 'f') independent of r2
 * (sep_spring_x0), and ends the program with sep_error otherwise. */
void sep_force_x0(seppart *ptr, char type, double (*fun)(double, char), sepsys *sys);
void sep_set_ndof(size_t ndof, sepsys *sys);
void sep_set_x0(seppart *ptr, int npart);
void sep_set_xn(seppart *ptr, int npart);

/* Number of linked-list cells along a box edge (reference :431). */
int sep_nsubbox(double cf, double delta, double lbox);
double sep_box_length(double dens, int npart, int ndim);

/* Mean momentum per degree of freedom (reference :434). */
double sep_eval_mom(seppart *ptr, int npart);

#endif
