/*
 * sep_api_gpu.c - the entry points this implementation adds (include/sepgpu.h).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "sep_rt.h"

void rt_pairset(rt_ctx *c, sepdev_pairset *ps);

int sep_gpu_available(void)
{
	return sepdev_device_count() > 0;
}

const char *sep_gpu_error(void)
{
	return sepdev_last_error();
}

int sep_gpu_sync(seppart *ptr)
{
	rt_ctx *c = rt_get(ptr, __func__);
	rt_need_host(c);
	return 0;
}

int sep_gpu_invalidate(seppart *ptr)
{
	rt_ctx *c = rt_get(ptr, __func__);
	rt_flush(c);
	c->host_valid = 1;
	c->dev_valid = 0;
	c->x0_valid = 0;
	c->forces_zero = 0;
	return 0;
}

int sep_gpu_set_tuning(const sep_gpu_tuning *t)
{
	if (!t || t->nclass < 1 || t->nclass > SEP_GPU_NCLASS) return -1;
	sepdev_tuning d;
	memset(&d, 0, sizeof d);
	d.nclass = t->nclass;
	for (int k = 0; k < t->nclass; k++) {
		d.nmax[k] = t->nmax[k];
		d.team[k] = t->team[k];
		d.groups[k] = t->groups[k];
		d.cellf[k] = t->cellf[k];
	}
	return sepdev_tuning_set(&d) == SEPDEV_OK ? 0 : -1;
}

int sep_gpu_get_tuning(sep_gpu_tuning *t)
{
	if (!t) return -1;
	sepdev_tuning d;
	sepdev_tuning_get(&d);
	memset(t, 0, sizeof *t);
	t->nclass = d.nclass;
	for (int k = 0; k < d.nclass; k++) {
		t->nmax[k] = d.nmax[k];
		t->team[k] = d.team[k];
		t->groups[k] = d.groups[k];
		t->cellf[k] = d.cellf[k];
	}
	return 0;
}

int sep_gpu_info_get(seppart *ptr, sep_gpu_info *info)
{
	rt_ctx *c = rt_get(ptr, __func__);
	memset(info, 0, sizeof *info);
	info->list_builds = c->nbuild;
	if (!c->dev) return 0;
	info->launches = sepdev_launch_count(c->dev);
	int mx = 0, cap = 0;
	double mean = 0.0;
	sepdev_list_stats(c->dev, &mx, &mean, &cap);   /* the last list built */
	info->list_capacity = cap;
	info->list_max = mx;
	info->list_mean = mean;
	sepdev_params(c->dev, &info->team, &info->groups, &info->cellf);
	info->direct_io = sepdev_direct_io(c->dev);
	return 0;
}

long sep_gpu_list_pairs(seppart *ptr, int *pairs, long cap)
{
	rt_ctx *c = rt_get(ptr, __func__);
	if (!c->dev || c->list_stale) return -1;
	return sepdev_list_pairs(c->dev, pairs, cap);
}

int sep_gpu_event_record(seppart *ptr, int e)
{
	rt_ctx *c = rt_get(ptr, __func__);
	if (!c->dev) return -1;
	return sepdev_event_record(c->dev, e);
}

int sep_gpu_event_elapsed(seppart *ptr, int e0, int e1, float *ms)
{
	rt_ctx *c = rt_get(ptr, __func__);
	if (!c->dev) return -1;
	return sepdev_event_elapsed(c->dev, e0, e1, ms);
}

int sep_gpu_stream_sync(seppart *ptr)
{
	rt_ctx *c = rt_get(ptr, __func__);
	if (!c->dev) return 0;
	return sepdev_sync(c->dev);
}

/* Set up the single pair term of a device loop, as the first iteration's
 * sep_force_pairs / sep_force_lj call would. */
static rt_ctx *loop_setup(seppart *ptr, sepsys *sys, const char *types,
			  double (*fun)(double, char), const double *ljparam, double cf,
			  unsigned opt, sepdev_pairset *ps)
{
	rt_ctx *c = rt_get(ptr, "sep_gpu_run");
	const double rc = fun ? cf : ljparam[0];
	if (rc > sys->cf) sep_error("cutoff for an interaction cannot be larger than maximum cutoff");
	rt_need_device(c, sys);
	rt_flush(c);
	rt_prepare_list(c, sys, opt, 1);
	/* one pending term describes the loop's pair force */
	rt_term *T = &c->terms[0];
	memset(T, 0, sizeof *T);
	if (fun) {
		T->rc = cf; T->eps = 1.0; T->sigma = 1.0; T->aw = 1.0;
		if (fun == sep_lj_shift) { T->kind = SEPDEV_POT_LJ; T->ushift = SEP_LJCF2; }
		else if (fun == sep_lj) { T->kind = SEPDEV_POT_LJ; }
		else if (fun == sep_wca) { T->kind = SEPDEV_POT_LJ; T->ushift = 1.0; }
		else sep_error("sep_gpu_run: only sep_lj, sep_lj_shift, sep_wca or LJ parameters");
	} else {
		T->kind = SEPDEV_POT_LJ;
		T->rc = ljparam[0]; T->eps = ljparam[1]; T->sigma = ljparam[2]; T->aw = ljparam[3];
		T->ushift = -4.0 * T->eps * (pow(T->sigma / T->rc, 12.) - T->aw * pow(T->sigma / T->rc, 6.));
	}
	T->t0 = types[0];
	T->t1 = types[1];
	c->nterms = 1;
	c->coul_on = 0;
	rt_pairset(c, ps);
	c->nterms = 0;
	return c;
}

/* results of a device loop into sys and ret, as after the last sep_leapfrog */
static void loop_finish(rt_ctx *c, sepsys *sys, sepret *ret, const double *s, long nsteps,
			long ntrig, int last_trig)
{
	sep_reset_retval(ret);
	ret->epot = s[SLOT_EPOT0];
	ret->ekin = 0.5 * s[SLOT_EKIN];
	const double *P = s + SLOT_POTP, *K = s + SLOT_KINP;
	const int map[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
	for (int k = 0; k < 3; k++)
		for (int kk = 0; kk < 3; kk++) {
			ret->pot_P[k][kk] = P[map[k][kk]];
			ret->kin_P[k][kk] = K[map[k][kk]];
		}
	sys->max_dist2 = s[SLOT_MAXD2];
	sys->nupdate_neighb += (unsigned)ntrig;
	sys->tnow += nsteps * sys->dt;
	if (last_trig) {
		sys->neighb_flag = 1;
		c->list_stale = 1;
		c->trigger_next = 1;
	} else if (sys->neighb_update != SEP_BRUTE && ntrig > 0) {
		sys->neighb_flag = 0;
	}
	c->pending_trigger = 0;
	c->host_valid = 0;
	c->forces_zero = 0;
	c->friction = 0;
}

int sep_gpu_run(seppart *ptr, sepsys *sys, sepret *ret, const char *types,
		double (*fun)(double, char), const double *ljparam, double cf, unsigned opt,
		int nh, double T0, double *alpha, double tau, long nsteps)
{
	if (nsteps <= 0) return 0;
	sepdev_pairset ps;
	rt_ctx *c = loop_setup(ptr, sys, types, fun, ljparam, cf, opt, &ps);
	sepdev_runcfg cfg;
	memset(&cfg, 0, sizeof cfg);
	cfg.dt = sys->dt;
	cfg.skin = sys->skin;
	cfg.nh = nh;
	cfg.T0 = T0;
	cfg.tau = tau;
	cfg.force_trigger = c->pending_trigger;
	if (!c->sumv2_valid) {
		rt_check(sepdev_sumv2(c->dev, &c->sumv2), "kinetic sum");
		c->sumv2_valid = 1;
	}
	double a = alpha ? *alpha : 0.0, last[SLOT_FIELDS];
	if (nh) {
		/* the first step's thermostat update, exactly as sep_nosehoover */
		const double ekin = 0.5 * c->sumv2 / sys->npart;
		const double temp = 0.666667 * ekin;
		a = a + sys->dt / (tau * tau) * (temp / T0 - 1.0);
	}
	long ntrig = 0;
	int lt = 0;
	rt_check(sepdev_run(c->dev, &ps, &cfg, nsteps, &a, &c->sumv2, last, &ntrig, &lt), "device loop");
	if (alpha && nh) *alpha = a;
	c->nbuild += ntrig;
	loop_finish(c, sys, ret, last, nsteps, ntrig, lt);
	return 0;
}

static double time_kernel_loop(seppart *ptr, sepsys *sys, sepret *ret, const char *types,
			       double (*fun)(double, char), const double *ljparam, double cf,
			       unsigned opt, int nh, double T0, double *alpha, double tau,
			       long nsteps, long flush, int observe);

int sep_gpu_run_timed(seppart *ptr, sepsys *sys, sepret *ret, const char *types,
		      double (*fun)(double, char), const double *ljparam, double cf, unsigned opt,
		      int nh, double T0, double *alpha, double tau, long nsteps, sep_gpu_timing *tm)
{
	if (!tm) return -1;
	sepdev_timing t;
	memset(&t, 0, sizeof t);
	t.flush_bytes = tm->flush_bytes;
	t.kernel_spans = tm->kernel_spans;
	if (nsteps <= 0) {
		tm->ms_steps = tm->ms_kernel = 0.0;
		tm->launches = tm->overflows = 0;
		return 0;
	}
	if (tm->kernel_spans == 2 && tm->flush_bytes > 0) return -1;
	if (tm->kernel_spans == 1) {
		/* stream events around host-launched steps: an event node inside
		 * a graph costs several microseconds, a stream event much less */
		double a0 = alpha ? *alpha : 0.0;
		tm->ms_kernel = time_kernel_loop(ptr, sys, ret, types, fun, ljparam, cf, opt, nh, T0,
						 &a0, tau, nsteps, tm->flush_bytes, tm->observe);
		if (alpha && nh) *alpha = a0;
		tm->ms_steps = 0.0;
		tm->launches = nsteps;
		tm->overflows = 0;
		return 0;
	}
	sepdev_pairset ps;
	rt_ctx *c = loop_setup(ptr, sys, types, fun, ljparam, cf, opt, &ps);
	sepdev_runcfg cfg;
	memset(&cfg, 0, sizeof cfg);
	cfg.dt = sys->dt;
	cfg.skin = sys->skin;
	cfg.nh = nh;
	cfg.T0 = T0;
	cfg.tau = tau;
	cfg.force_trigger = c->pending_trigger;
	cfg.observe_all = tm->observe ? 1 : 0;
	if (!c->sumv2_valid) {
		rt_check(sepdev_sumv2(c->dev, &c->sumv2), "kinetic sum");
		c->sumv2_valid = 1;
	}
	double a = alpha ? *alpha : 0.0, last[SLOT_FIELDS];
	if (nh) {
		const double ekin = 0.5 * c->sumv2 / sys->npart;
		const double temp = 0.666667 * ekin;
		a = a + sys->dt / (tau * tau) * (temp / T0 - 1.0);
	}
	long ntrig = 0;
	int lt = 0;
	rt_check(sepdev_run_timed(c->dev, &ps, &cfg, nsteps, &a, &c->sumv2, last, &ntrig, &lt, &t),
		 "timed device loop");
	if (alpha && nh) *alpha = a;
	c->nbuild += ntrig + t.overflows;
	loop_finish(c, sys, ret, last, nsteps, ntrig, lt);
	tm->ms_steps = t.ms_steps;
	tm->ms_kernel = t.ms_kernel;
	tm->launches = t.launches;
	tm->overflows = t.overflows;
	return 0;
}

int sep_gpu_flush_l2(seppart *ptr, long bytes)
{
	rt_ctx *c = rt_find(ptr);
	if (!c || !c->dev || bytes <= 0) return -1;
	rt_check(sepdev_flush_l2(c->dev, (size_t)bytes, 7u), "L2 flush");
	rt_check(sepdev_sync(c->dev), "L2 flush");
	return 0;
}

/* the prgs loop one step at a time from the host, with events around each
 * fused step kernel; list rebuilds and (flush > 0) an L2 flush before each
 * step stay outside the events.  Returns the summed kernel time in ms. */
static double time_kernel_loop(seppart *ptr, sepsys *sys, sepret *ret, const char *types,
			       double (*fun)(double, char), const double *ljparam, double cf,
			       unsigned opt, int nh, double T0, double *alpha, double tau,
			       long nsteps, long flush, int observe)
{
	double total = 0.0;
	for (long s = 0; s < nsteps; s++) {
		sepdev_pairset ps;
		rt_ctx *c = loop_setup(ptr, sys, types, fun, ljparam, cf, opt, &ps);
		if (nh) {
			const double ekin = 0.5 * c->sumv2 / sys->npart;
			const double temp = 0.666667 * ekin;
			*alpha = *alpha + sys->dt / (tau * tau) * (temp / T0 - 1.0);
		}
		const int slot = rt_new_slot(c), lf = rt_new_slot(c);
		if (flush > 0) rt_check(sepdev_flush_l2(c->dev, (size_t)flush, (unsigned)s), "L2 flush");
		rt_check(sepdev_event_record(c->dev, 0), "event");
		/* as in the device loop, only the last step reports energy and
		 * virial, unless every step is to be observed */
		rt_check(sepdev_step_obs(c->dev, &ps, 0, sys->dt, nh, nh ? *alpha : 0.0, slot, lf,
					 observe || s + 1 == nsteps), "step");
		rt_check(sepdev_event_record(c->dev, 1), "event");
		float ms = 0.f;
		rt_check(sepdev_event_elapsed(c->dev, 0, 1, &ms), "event");
		total += ms;
		sep_reset_retval(ret);
		rt_add_op(c, ret, OP_PAIR_ASSIGN, slot, 0);
		rt_add_op(c, ret, OP_VIRIAL, slot, 0);
		rt_add_op(c, ret, OP_KIN, lf, 0);
		sys->max_dist2 = 0.0;
		rt_read_slots(c, sys, lf);
		if (sqrt(sys->max_dist2) > sys->skin * 0.5 || c->pending_trigger) {
			sys->neighb_flag = 1;
			sys->nupdate_neighb++;
			c->list_stale = 1;
			c->trigger_next = 1;
			c->pending_trigger = 0;
		}
		sys->tnow += sys->dt;
		c->host_valid = 0;
		c->forces_zero = 0;
	}
	return total;
}

int sep_gpu_time_step_kernel(seppart *ptr, sepsys *sys, sepret *ret, const char *types,
			     double (*fun)(double, char), const double *ljparam, double cf,
			     unsigned opt, int nh, double T0, double *alpha, double tau,
			     long nsteps, double *ms_per_launch)
{
	const double total = time_kernel_loop(ptr, sys, ret, types, fun, ljparam, cf, opt, nh, T0,
					       alpha, tau, nsteps, 0, 0);
	if (ms_per_launch) *ms_per_launch = nsteps > 0 ? total / nsteps : 0.0;
	return 0;
}
