/*
 * sepret.h - return-value helpers (reference include/sepret.h:36-61).
 */
#ifndef SEP_GB300_SEPRET_H
#define SEP_GB300_SEPRET_H

#include <stdio.h>
#include <math.h>
#include <stdlib.h>
#include "sepstrct.h"

/* Zeroes energies and tensors (reference :36). */
void sep_reset_retval(sepret *retval);
/* Normal pressure, after filling P (reference :44). */
double sep_get_pressure(sepret *retval, sepsys *sys);
/* 2 ekin / (3 ndof) (reference :52). */
double sep_get_temperature(sepret *retval, sepsys *sys);
/* P = (kin_P + pot_P)/V and p = tr(P)/3 (reference :61). */
void sep_pressure_tensor(sepret *retval, sepsys *sys);

/*
 * Molecular pressure tensor (reference :67, source/sepret.c:85-102,
 * source/sepmol.c:913-959): kin_P_mol = sum M v_cm v_cm^T,
 * pot_P_mol = sum_{i<j} F_ij (x) R_ij over the intermolecular forces of the
 * pair calls since sep_reset_force_mol and the centres of mass now;
 * P_mol = (kin_P_mol + pot_P_mol)/V, p_mol = tr P_mol / 3.  mol[i].x and
 * mol[i].v receive the centres of mass and their velocities.  Needs
 * sep_init_mol (flag_Fij); without it only P_mol and p_mol are formed from
 * the values already in retval.
 */
void sep_mol_pressure_tensor(sepatom *atoms, sepmol *mols, sepret *retval, sepsys *sys);

#endif
