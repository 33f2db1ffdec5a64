/*
 * sepmol.h - molecular topology and bonded forces
 * (reference include/sepmol.h:18-100).
 */
#ifndef SEP_GB300_SEPMOL_H
#define SEP_GB300_SEPMOL_H

#include <stdio.h>
#include "sepdef.h"
#include "sepstrct.h"
#include "sepmisc.h"

/* Reads the [ bonds ], [ angles ] and [ dihedrals ] sections of a topology
 * file, filling the lists, molindex and the exclusion arrays (reference :18). */
void sep_read_topology_file(sepatom *aptr, const char *file, sepsys *sys, char opt);

/* Harmonic bond U = k/2 (r - l0)^2 for bonds of `type` (reference :31). */
void sep_stretch_harmonic(sepatom *aptr, int type, const double lbond,
			  const double ks, sepsys *sys, sepret *ret);

/* Cosine-squared angle U = k/2 (cos(pi - theta) - cos(pi - angle0))^2 (reference :57). */
void sep_angle_cossq(sepatom *ptr, int type, const double angle0,
		     const double k, sepsys *sys, sepret *ret);

/* Harmonic angle U = k/2 (theta - angle0)^2 (reference :70). */
void sep_angle_harmonic(sepatom *ptr, int type, const double angle0,
			const double k, sepsys *sys, sepret *ret);

/* Ryckaert-Bellemans torsion U = sum_n g[n] cos^n psi (reference :83). */
void sep_torsion_Ryckaert(sepatom *ptr, int type, const double g[6],
			  sepsys *sys, sepret *ret);

/* Molecule table from molindex (reference :93) and its release (reference :100). */
sepmol *sep_init_mol(sepatom *atom, sepsys *sys);
void sep_free_mol(sepmol *ptr, sepsys *sys);

/* Centre of mass of every molecule into mol[i].x (the chain of consecutive
 * atoms from its first one, bonds unwrapped, wrapped into the box) and
 * centre-of-mass velocity into mol[i].v (source/sepmol.c:683-748). */
void sep_mol_cm(seppart *ptr, sepmol *mol, sepsys *sys);
void sep_mol_velcm(seppart *atom, sepmol *mol, sepsys *sys);

/* Section readers and list release (reference :212-219). */
void sep_read_bonds_top(sepatom *aptr, sepmolinfo *ptr, const char *file, int npart, char opt);
void sep_read_angles_top(sepatom *aptr, sepmolinfo *ptr, const char *file, int npart, char opt);
void sep_read_dihedrals_top(sepatom *aptr, sepmolinfo *ptr, const char *file, int npart, char opt);
void sep_free_bonds(sepmolinfo *ptr);
void sep_free_angles(sepmolinfo *ptr);
void sep_free_dihedrals(sepmolinfo *ptr);

#endif
