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

#endif
