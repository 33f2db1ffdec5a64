/*
 * sep_api_intgr.c - Nose-Hoover thermostat and leap-frog of the sep C API.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "sep_rt.h"

/* Nose-Hoover (source/sepintgr.c:149-168).  The thermostat update itself is
 * scalar and done here in FP64 from the device's exact sum m v^2 (made
 * current first: a program that changed the particles on the host has them
 * uploaded here); the friction f -= alpha m v is deferred to the next force
 * materialisation, normally the fused leap-frog kernel. */
void sep_nosehoover(seppart *ptr, double temp0, double *alpha, const double tau, sepsys *sys)
{
	rt_ctx *c = rt_get(ptr, __func__);
	rt_need_device(c, sys);
	if (!c->sumv2_valid) {
		rt_check(sepdev_sumv2(c->dev, &c->sumv2), "kinetic sum");
		c->sumv2_valid = 1;
	}
	const double ekin = 0.5 * c->sumv2 / sys->npart;
	const double temp = 0.666667 * ekin;
	*alpha = *alpha + sys->dt / (tau * tau) * (temp / temp0 - 1.0);
	c->friction = 1;
	c->friction_alpha += *alpha;
	c->host_valid = 0;
}

/* Leap-frog (source/sepintgr.c:42-88).  Pending pair terms, friction and the
 * integration run as one fused kernel; the step's sums are read back and
 * applied to retval and sys before returning, so the program sees the
 * reference's values after every call. */
void sep_leapfrog(seppart *ptr, sepsys *sys, sepret *retval)
{
	rt_ctx *c = rt_get(ptr, __func__);
	rt_need_device(c, sys);
	int lf;
	/* pending bonded terms go first; the step adds the pair forces to them */
	rt_launch_bonded(c);
	sepdev_pairset ps;
	int fused = 0, acc = 0, fr = 0, pslot = -1;
	double fa = 0.0;
	if (c->pass_slot >= 0) {
		extern void rt_pairset(rt_ctx *c, sepdev_pairset *ps);
		rt_pairset(c, &ps);
		rt_pass_mol_slot(c);
		lf = rt_new_slot(c);
		fused = 1;
		acc = !c->forces_zero;
		fr = c->friction;
		fa = c->friction_alpha;
		pslot = c->pass_slot;
		rt_check(sepdev_step_deferred(c->dev, &ps, acc, sys->dt, fr, fa, pslot, lf, c->nslots),
			 "fused step");
		c->nterms = 0;
		c->coul_on = 0;
		c->pass_slot = -1;
	} else {
		if (c->forces_zero) rt_check(sepdev_zero_forces(c->dev), "force reset");
		lf = rt_new_slot(c);
		rt_check(sepdev_leapfrog(c->dev, sys->dt, c->friction, c->friction_alpha, lf), "leap-frog");
	}
	c->forces_zero = 0;
	c->friction = 0;
	c->friction_alpha = 0.0;
	c->host_valid = 0;
	rt_add_op(c, retval, OP_KIN, lf, 0);
	if (fused) {
		/* the list built in this step's sep_force_pairs overflowed: the
		 * step did nothing; grow the list and run it again */
		while (rt_read_step_slots(c, sys, lf)) {
			sepdev_step_retract(c->dev);
			rt_check(sepdev_list_confirm(c->dev), "neighbour-list build");
			rt_pass_mol_slot(c);
			rt_check(sepdev_step_deferred(c->dev, &ps, acc, sys->dt, fr, fa, pslot, lf, c->nslots),
				 "fused step");
		}
	} else {
		rt_read_slots(c, sys, lf);
	}
	if (sqrt(sys->max_dist2) > sys->skin * 0.5 || c->pending_trigger) {
		sys->neighb_flag = 1;
		sys->nupdate_neighb++;
		c->list_stale = 1;
		c->trigger_next = 1;
		c->pending_trigger = 0;
	}
	sys->tnow += sys->dt;
}
