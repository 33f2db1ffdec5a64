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

/*
 * Groot-Warren (DPD) velocity Verlet: a = f/m; v += dt (a + pa)/2 unless
 * stepnow is 0; x += v dt + a dt^2/2; pv = v + lambda dt a; pa = a;
 * ret->ekin and ret->kin_P accumulate from the updated v.  Crossing the skin
 * raises sys->neighb_flag without counting an update, as the reference does
 * (reference :78, source/sepintgr.c:296-345).
 */
void sep_verlet_dpd(seppart *ptr, double lambda, int stepnow, sepsys *sys, sepret *retval);

/*
 * Fokker-Planck (Brownian) step with friction T/ldiff per particle:
 * x += v dt; v += dt/m (f - fric v + g sqrt(2 T fric/dt)), g standard normal
 * (reference :68, source/sepintgr.c:235-293).
 */
void sep_fp(seppart *ptr, double temp_desired, sepsys *sys, sepret *retval);

/*
 * Langevin step of Gronbech-Jensen and Farago with friction alpha; keeps the
 * previous force and Gaussian draw in prevf and randn; advances sys->tnow
 * (reference :46, source/sepintgr.c:91-146).
 */
void sep_langevinGJF(sepatom *ptr, double temp0, double alpha, sepsys *sys, sepret *retval);

#endif
