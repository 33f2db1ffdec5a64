/*
 * sep_api_typeops.c - per-type operations of the sep C API: the tether
 * force towards the initial positions (sep_force_x0, reference
 * source/sepmisc.c:645-670), the temperature relaxation of one type
 * (sep_relax_temp, :357-391) and the momentum reset of one type
 * (sep_reset_momentum, :1173-1192).  With the particles on the device they
 * run there (dev_typeops.cu); the scalar arithmetic between the sums and the
 * update is the reference's, in FP64 on the host.
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include "sep_rt.h"

/* source/sepmisc.c:645-670.  The device evaluates linear tethers: fun(r2,
 * 'f') must not depend on r2 (sep_spring_x0 and any spring of that form).
 * The reference computes the tether energy without storing it anywhere;
 * so does this. */
void sep_force_x0(seppart *ptr, char type, double (*fun)(double, char), sepsys *sys)
{
	rt_ctx *c = rt_get(ptr, __func__);
	const double ft = fun(1.0, 'f');
	if (fun(0.0, 'f') != ft || fun(0.25, 'f') != ft || fun(4.0, 'f') != ft)
		sep_error("%s: only linear tethers (fun(r2, 'f') independent of r2, as sep_spring_x0) "
			  "are provided by this GPU implementation", __func__);
	rt_need_device(c, sys);
	if (!c->x0_valid) {
		double *x0 = malloc(sizeof(double) * 3 * (c->n > 0 ? c->n : 1));
		if (!x0) sep_error("%s: couldn't allocate memory", __func__);
		for (long i = 0; i < c->n; i++)
			for (int k = 0; k < 3; k++) x0[3 * i + k] = ptr[i].x0[k];
		rt_check(sepdev_set_x0(c->dev, x0), "tether positions");
		free(x0);
		c->x0_valid = 1;
	}
	const int tid = rt_type_id(c, type);
	rt_materialize_forces(c);
	if (tid >= 0) rt_check(sepdev_tether(c->dev, tid, -ft), "tether force");
	c->host_valid = 0;
}

/* v = v fact - shift over the type: the device path of the two calls below */
static int type_update(rt_ctx *c, char type, int relax, double Td, double tau, sepsys *sys)
{
	if (!(c->dev && c->dev_valid)) return 0;
	const int tid = rt_type_id(c, type);
	double s[6] = {0, 0, 0, 0, 0, 0};
	if (tid >= 0) rt_check(sepdev_type_sums(c->dev, tid, s), "type sums");
	double fact = 1.0;
	if (relax) {
		const double ekin = 0.5 * s[4];
		if (ekin < DBL_EPSILON)
			sep_warning("%s: Zero kinetic energy - check your the types.", "sep_relax_temp");
		const double Ta = 2.0 * ekin / (3 * s[5]);
		fact = sqrt(1.0 + (sys->dt / tau) * (Td / Ta - 1.0));
	}
	/* the momentum of the scaled velocities over the type's mass */
	double shift[3] = {0, 0, 0};
	if (s[3] > 0.0)
		for (int k = 0; k < 3; k++) shift[k] = fact * s[k] / s[3];
	if (tid >= 0) rt_check(sepdev_type_scale(c->dev, tid, fact, shift), "velocity update");
	c->host_valid = 0;
	c->sumv2_valid = 0;
	return 1;
}

void sep_reset_momentum(seppart *ptr, const char type, sepsys *sys)
{
	rt_ctx *c = rt_get(ptr, __func__);
	if (type_update(c, type, 0, 0.0, 1.0, sys)) return;
	rt_host_modified(c);
	double mom[3] = {0, 0, 0}, mass = 0.0;
	for (long i = 0; i < sys->npart; i++)
		if (ptr[i].type == type) {
			for (int k = 0; k < 3; k++) mom[k] += ptr[i].v[k] * ptr[i].m;
			mass += ptr[i].m;
		}
	for (long i = 0; i < sys->npart; i++)
		if (ptr[i].type == type)
			for (int k = 0; k < 3; k++) ptr[i].v[k] -= mom[k] / mass;
}

void sep_relax_temp(seppart *ptr, char type, double Td, double tau, sepsys *sys)
{
	rt_ctx *c = rt_get(ptr, __func__);
	if (type_update(c, type, 1, Td, tau, sys)) return;
	rt_host_modified(c);
	double ekin = 0.0;
	int ntype = 0;
	for (long n = 0; n < sys->npart; n++)
		if (ptr[n].type == type) {
			ntype++;
			for (int k = 0; k < 3; k++) ekin += ptr[n].m * ptr[n].v[k] * ptr[n].v[k];
		}
	ekin = 0.5 * ekin;
	if (ekin < DBL_EPSILON) sep_warning("%s: Zero kinetic energy - check your the types.", __func__);
	const double Ta = 2.0 * ekin / (3 * ntype);
	const double fact = sqrt(1.0 + (sys->dt / tau) * (Td / Ta - 1.0));
	for (long n = 0; n < sys->npart; n++)
		if (ptr[n].type == type)
			for (int k = 0; k < 3; k++) ptr[n].v[k] *= fact;
	sep_reset_momentum(ptr, type, sys);
}
