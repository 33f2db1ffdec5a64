/*
 * sep_api_stoch.c - stochastic dynamics of the sep C API: the DPD pair force
 * of Groot and Warren, their velocity-Verlet integrator, the Fokker-Planck
 * and GJF Langevin integrators, and sep_set_ldiff.
 *
 * The reference draws its random numbers from rand() in loop order.  This
 * library draws them from counter-based streams (dev_stoch.cu): the same
 * distributions (uniform of unit variance per DPD pair, standard normal per
 * integrator coordinate), other individual values.  sep_gpu_set_seed
 * chooses the key.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include "sep_rt.h"

int sep_gpu_set_seed(seppart *ptr, unsigned long long seed)
{
	rt_ctx *c = rt_get(ptr, __func__);
	c->seed = seed;
	for (int k = 0; k < 4; k++) c->ncall[k] = 0;
	return 0;
}

/* source/sepprfrc.c:284-290 */
static void brute_omp_reset(sepsys *sys)
{
	if (sys->neighb_update == SEP_BRUTE && sys->omp_flag) {
		sep_warning("omp flag set, SEP_BRUTE does not support threads.");
		sep_warning("Resetting omp flag");
		sys->omp_flag = false;
	}
}

static void dpd(const char *caller, seppart *ptr, const char *types, double cf, double aij,
		double temp, double sigma, sepsys *sys, sepret *ret, unsigned opt, int brute)
{
	rt_ctx *c = rt_get(ptr, caller);
	rt_need_ext(c, sys);
	if (brute) {
		/* every pair within cf, no exclusions (source/sepprfrc.c:1134-1235) */
		if (cf > c->brute_cf) c->brute_cf = cf;
		rt_prepare_list(c, sys, SEP_ALL, 0);
	} else {
		rt_prepare_list(c, sys, opt, 1);
	}
	/* the forces the DPD pass adds to must exist first; a reset that is
	 * still pending is folded into the pass */
	int accumulate = 1;
	if (c->forces_zero && c->pass_slot < 0 && c->nbq == 0 && !c->friction) {
		accumulate = 0;
		c->forces_zero = 0;
	} else {
		rt_materialize_forces(c);
	}
	/* the O(N^2) form adds its conservative forces to the molecular tensor
	 * (source/sepprfrc.c:1211-1222) */
	const int molv = brute && c->mv_on && c->mv_uploaded;
	if (c->nslots >= (molv ? 13 : 14)) rt_flush(c);
	const int slot = rt_new_slot(c), slot2 = brute ? rt_new_slot(c) : -1;
	const int mslot = molv ? rt_new_slot(c) : -1;
	sepdev_dpd p;
	p.tA = rt_type_id(c, types[0]);
	p.tB = rt_type_id(c, types[1]);
	p.cf = cf; p.aij = aij; p.sigma = sigma; p.dt = sys->dt;
	p.gamma = sigma * sigma / (2.0 * temp);
	p.seed = c->seed;
	p.call = c->ncall[RT_STREAM_DPD]++;
	p.virial = brute;
	p.mslot = mslot;
	rt_check(sepdev_dpd_forces(c->dev, &p, accumulate, slot, slot2), "DPD forces");
	rt_add_op(c, ret, brute ? OP_PAIR_ADD : OP_PAIR_ASSIGN, slot, 0);
	if (brute) rt_add_op(c, ret, OP_DPD_VIR, slot, slot2);
	if (molv) rt_add_op(c, NULL, OP_MOLVIR, mslot, 0);
	c->host_valid = 0;
}

/* source/sepprfrc.c:278-301 */
void sep_force_dpd(seppart *ptr, const char *types, const double cf, const double aij,
		   const double temp_desired, const double sigma, sepsys *sys, sepret *retval,
		   const unsigned opt)
{
	const int brute = sys->neighb_update == SEP_BRUTE;
	if (brute) brute_omp_reset(sys);
	dpd(__func__, ptr, types, cf, aij, temp_desired, sigma, sys, retval, opt, brute);
}

/* source/sepprfrc.c:1007-1104 */
void sep_dpdforce_neighb(seppart *ptr, const char *types, const double cf, const double aij,
			 const double temp_desired, const double sigma, sepsys *sys,
			 sepret *retval, const unsigned opt)
{
	dpd(__func__, ptr, types, cf, aij, temp_desired, sigma, sys, retval, opt, 0);
}

/* source/sepprfrc.c:1134-1235 */
void sep_dpdforce_brute(seppart *ptr, const char *types, const double cf, const double aij,
			const double temp_desired, const double sigma, sepsys *sys,
			sepret *retval)
{
	dpd(__func__, ptr, types, cf, aij, temp_desired, sigma, sys, retval, SEP_ALL, 1);
}

/* integrator epilogue: kinetic sums into retval, the skin test */
static void finish_step(rt_ctx *c, sepsys *sys, sepret *ret, int lf, int count_update)
{
	c->host_valid = 0;
	rt_add_op(c, ret, OP_KIN, lf, 0);
	rt_read_slots(c, sys, lf);
	if (sqrt(sys->max_dist2) > sys->skin * 0.5 || c->pending_trigger) {
		sys->neighb_flag = 1;
		if (count_update) sys->nupdate_neighb++;
		c->list_stale = 1;
		c->trigger_next = 1;
		c->pending_trigger = 0;
	}
}

/* source/sepintgr.c:296-345 (no update count, no tnow advance) */
void sep_verlet_dpd(seppart *ptr, double lambda, int stepnow, sepsys *sys, sepret *retval)
{
	rt_ctx *c = rt_get(ptr, __func__);
	rt_need_ext(c, sys);
	rt_materialize_forces(c);
	const int lf = rt_new_slot(c);
	rt_check(sepdev_verlet_dpd(c->dev, sys->dt, lambda, stepnow, lf), "Groot-Warren step");
	finish_step(c, sys, retval, lf, 0);
}

/* source/sepintgr.c:235-293 (counts the update, no tnow advance) */
void sep_fp(seppart *ptr, double temp_desired, sepsys *sys, sepret *retval)
{
	rt_ctx *c = rt_get(ptr, __func__);
	rt_need_ext(c, sys);
	rt_materialize_forces(c);
	const int lf = rt_new_slot(c);
	rt_check(sepdev_fp(c->dev, sys->dt, temp_desired, c->seed, c->ncall[RT_STREAM_FP]++, lf),
		 "Fokker-Planck step");
	finish_step(c, sys, retval, lf, 1);
}

/* source/sepintgr.c:91-146 (counts the update, advances tnow) */
void sep_langevinGJF(sepatom *ptr, double temp0, double alpha, sepsys *sys, sepret *retval)
{
	rt_ctx *c = rt_get(ptr, __func__);
	rt_need_ext(c, sys);
	rt_materialize_forces(c);
	const int lf = rt_new_slot(c);
	rt_check(sepdev_gjf(c->dev, sys->dt, temp0, alpha, c->seed, c->ncall[RT_STREAM_GJF]++, lf),
		 "GJF Langevin step");
	finish_step(c, sys, retval, lf, 1);
	sys->tnow += sys->dt;
}

/* source/sepmisc.c:1162-1170 */
void sep_set_ldiff(seppart *ptr, char type, double ldiff, sepsys sys)
{
	rt_ctx *c = rt_find(ptr);
	if (c && c->dev) rt_host_modified(c);
	for (long n = 0; n < sys.npart; n++)
		if (ptr[n].type == type) ptr[n].ldiff = ldiff;
}
