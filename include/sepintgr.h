/*
 * sepintgr.h - integrator and thermostat (reference include/sepintgr.h:35-58).
 */
#ifndef SEP_GB300_SEPINTGR_H
#define SEP_GB300_SEPINTGR_H

#include "sepmisc.h"
#include "sepstrct.h"

/*
 * Leap-frog step: a = f/m, v += a dt, x += v dt, periodic wrap with crossing
 * counts; ret->ekin and ret->kin_P accumulate from v - a dt/2; a neighbour
 * list update is flagged when the largest displacement since the last update
 * exceeds skin/2 (reference :35, source/sepintgr.c:18-88).
 */
void sep_leapfrog(seppart *ptr, sepsys *sys, sepret *retval);

/*
 * Nose-Hoover friction: T = 0.666667 * (sum m v^2 / 2N),
 * alpha += dt/Q^2 (T/Td - 1), f -= alpha m v (reference :58,
 * source/sepintgr.c:149-168).
 */
void sep_nosehoover(seppart *ptr, double Td, double *alpha, const double Q,
		    sepsys *sys);

#endif
