/*
 * sep_api_init.c - set-up, input/output, return values and small helpers of
 * the sep C API.  Each function states the reference function whose
 * behaviour it reproduces.
 */
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "sep_rt.h"

/* host neighbour arrays are not used: every particle points at this one
 * terminated list, so a program that walks atoms[i].neighb sees no entries */
static int g_no_neighb[1] = {-1};

/* ---- messages (source/sepmisc.c:16-113) ---------------------------------------- */

void sep_error(char *str, ...)
{
	va_list ap;
	printf("sep-error -> ");
	va_start(ap, str);
	vprintf(str, ap);
	va_end(ap);
	printf("\nBAILING OUT\n");
	fflush(stdout);
	exit(EXIT_FAILURE);
}

void sep_warning(char *str, ...)
{
	va_list ap;
	printf("sep-warning -> ");
	va_start(ap, str);
	vprintf(str, ap);
	va_end(ap);
	printf("\n");
	fflush(stdout);
}

/* ---- allocation (source/sepinit.c:16-65) ------------------------------------------ */

seppart *sep_init(size_t npart, size_t nneighb)
{
	(void)nneighb;
	if (npart == 0) sep_error("%s: zero particles", __func__);
	seppart *p = calloc(npart, sizeof(seppart));
	if (!p) sep_error("%s at line %d: Couldn't allocate memory\n", __func__, __LINE__);
	for (size_t i = 0; i < npart; i++) {
		p[i].type = 'A';
		p[i].m = 1.0;
		p[i].molindex = -1;
		p[i].ldiff = 1.0;
		p[i].neighb = g_no_neighb;
		for (int k = 0; k < SEP_BOND; k++) p[i].bond[k] = -1;
		for (int k = 0; k < SEP_ANGLE; k++) p[i].angle[k] = -1;
		for (int k = 0; k < SEP_DIHED; k++) p[i].dihed[k] = -1;
	}
	rt_register(p, (long)npart);
	return p;
}

void sep_close(seppart *ptr, size_t npart)
{
	(void)npart;
	if (!ptr) return;
	rt_unregister(ptr);
	free(ptr);
}

/* xyz reader (source/sepinit.c:69-109): count, box, then
 * "type x y z vx vy vz m z" per particle */
seppart *sep_init_xyz(double *lbox, int *npart, const char *file, char verbose)
{
	if (verbose == 'v') fprintf(stdout, "Opening %s\n", file);
	FILE *fin = fopen(file, "r");
	if (!fin) sep_error("%s at line %d: Couldn't open file\n", __func__, __LINE__);
	if (fscanf(fin, "%d", npart) != 1 || *npart <= 0)
		sep_error("%s at line %d: Error reading xyz file\n", __func__, __LINE__);
	seppart *p = sep_init((size_t)*npart, SEP_NUM_NEIGHB);
	if (fscanf(fin, "%lf%lf%lf\n", &lbox[0], &lbox[1], &lbox[2]) != 3)
		sep_error("%s at line %d: Error reading xyz file\n", __func__, __LINE__);
	for (int i = 0; i < *npart; i++)
		if (fscanf(fin, "%c%lf%lf%lf%lf%lf%lf%lf%lf\n", &p[i].type, &p[i].x[0], &p[i].x[1],
			   &p[i].x[2], &p[i].v[0], &p[i].v[1], &p[i].v[2], &p[i].m, &p[i].z) != 9)
			sep_error("%s at line %d: Error reading xyz file\n", __func__, __LINE__);
	if (verbose == 'v') {
		fprintf(stdout, "Closing file\nNumber of particles: %d\n", *npart);
		fflush(stdout);
	}
	fclose(fin);
	return p;
}

/* ---- system (source/sepinit.c:246-314, source/sepmisc.c:1116-1129) -------------------- */

int sep_nsubbox(double cf, double delta, double lbox)
{
	return (int)(lbox / (cf + delta));
}

double sep_box_length(double dens, int npart, int ndim)
{
	return pow((double)npart / dens, 1.0 / ndim);
}

sepsys sep_sys_setup(double lx, double ly, double lz, double cf, double dt, size_t npart,
		     size_t update)
{
	sepsys s;
	const double skin = 0.25;   /* the reference's fixed set-up skin */
	memset(&s, 0, sizeof s);
	s.length[0] = lx; s.length[1] = ly; s.length[2] = lz;
	s.volume = lx * ly * lz;
	const char axis[3] = {'x', 'y', 'z'};
	for (int k = 0; k < 3; k++) {
		s.nsubbox[k] = sep_nsubbox(cf, skin, s.length[k]);
		if (update > 1 && s.nsubbox[k] < 3)
			sep_warning("%s at %d: Number of subboxes in %c direction are less than three",
				    __func__, __LINE__, axis[k]);
		s.lsubbox[k] = s.length[k] / s.nsubbox[k];
	}
	s.npart = (long)npart;
	s.cf = cf;
	s.dt = dt;
	s.ndof = 3 * (unsigned)npart - 3;
	s.tnow = 0.0;
	s.nupdate_neighb = 0;
	s.neighb_update = (unsigned)update;
	s.neighb_flag = 1;
	s.skin = skin;
	s.molptr = calloc(1, sizeof(sepmolinfo));
	if (!s.molptr) sep_error("%s at line %d: Couldn't allocate memory", __func__, __LINE__);
	s.molptr->flag_Fij = 0;
	s.omp_flag = false;
	s.fun_cstate = 0;
	return s;
}

void sep_free_sys(sepsys *sys)
{
	sep_free_bonds(sys->molptr);
	sep_free_angles(sys->molptr);
	sep_free_dihedrals(sys->molptr);
}

void sep_set_omp(unsigned nthreads, sepsys *sys)
{
	sys->omp_flag = true;
	sys->nthreads = nthreads;
}

void sep_set_skin(sepsys *sys, double value)
{
	sys->skin = value;
}

void sep_set_ndof(size_t ndof, sepsys *sys)
{
	sys->ndof = (unsigned)ndof;
}

/* ---- initial state (source/sepinit.c:113-244, :317-352) ----------------------------- */

void sep_set_lattice(seppart *ptr, sepsys sys)
{
	rt_ctx *c = rt_get(ptr, __func__);
	rt_host_modified(c);
	const double dens = sys.npart / (sys.length[0] * sys.length[1] * sys.length[2]);
	int numb[3];
	double gap[3];
	for (int k = 0; k < 3; k++) {
		numb[k] = (int)ceil(pow(dens, 1. / 3.) * sys.length[k]);
		gap[k] = sys.length[k] / numb[k];
	}
	long n = 0;
	for (int iz = 0; iz < numb[2]; iz++)
		for (int iy = 0; iy < numb[1]; iy++)
			for (int ix = 0; ix < numb[0]; ix++) {
				ptr[n].x[0] = ix * gap[0] + 1.0;
				ptr[n].x[1] = iy * gap[1] + 1.0;
				ptr[n].x[2] = iz * gap[2] + 1.0;
				if (++n == sys.npart) return;
			}
}

/* uniform velocities U(-1/2, 1/2) from rand(), centre-of-mass momentum
 * removed, scaled to sum m v^2 = 3 N T, then the two extra draws per
 * component the reference spends on its DPD predictors, so the rand()
 * stream after the call is the reference's */
static void set_vel_common(seppart *p, double temp, long n, int keep_noise)
{
	double mom[3] = {0, 0, 0}, ek = 0.0;
	for (long i = 0; i < n; i++)
		for (int k = 0; k < 3; k++) {
			p[i].v[k] = sep_rand() - 0.5;
			mom[k] += p[i].v[k] * p[i].m;
			ek += p[i].v[k] * p[i].v[k] * p[i].m;
		}
	const double scale = sqrt(3.0 * n * temp / ek);
	for (long i = 0; i < n; i++)
		for (int k = 0; k < 3; k++) p[i].v[k] = (p[i].v[k] - mom[k] / (p[i].m * n)) * scale;
	for (long i = 0; i < n; i++)
		for (int k = 0; k < 3; k++) {
			double nx = (sep_rand() - 0.5) * 0.01, nv = (sep_rand() - 0.5) * 0.01;
			p[i].px[k] = p[i].x[k] + (keep_noise ? nx : 0.0);
			p[i].pv[k] = p[i].v[k] + (keep_noise ? nv : 0.0);
			if (!keep_noise) p[i].pa[k] = 0.0;
		}
}

void sep_set_vel(seppart *ptr, double temp, sepsys sys)
{
	rt_ctx *c = rt_get(ptr, __func__);
	rt_host_modified(c);
	srand((unsigned)time(NULL));
	set_vel_common(ptr, temp, sys.npart, 1);
}

void sep_set_vel_seed(seppart *ptr, double temp, unsigned int seed, sepsys sys)
{
	rt_ctx *c = rt_get(ptr, __func__);
	rt_host_modified(c);
	srand(seed);
	set_vel_common(ptr, temp, sys.npart, 0);
}

void sep_set_vel_type(seppart *ptr, char type, double temp, unsigned int seed, sepsys sys)
{
	rt_ctx *c = rt_get(ptr, __func__);
	rt_host_modified(c);
	const long n = sys.npart;
	const int ntype = sep_count_type(ptr, type, (int)n);
	if (ntype == 0) return;
	srand(seed);
	double mom[3] = {0, 0, 0}, ek = 0.0;
	for (long i = 0; i < n; i++)
		if (ptr[i].type == type)
			for (int k = 0; k < 3; k++) {
				ptr[i].v[k] = sep_rand() - 0.5;
				mom[k] += ptr[i].v[k] * ptr[i].m;
				ek += ptr[i].v[k] * ptr[i].v[k] * ptr[i].m;
			}
	const double scale = sqrt(3.0 * ntype * temp / ek);
	for (long i = 0; i < n; i++)
		if (ptr[i].type == type)
			for (int k = 0; k < 3; k++)
				ptr[i].v[k] = (ptr[i].v[k] - mom[k] / (ptr[i].m * ntype)) * scale;
	for (long i = 0; i < n; i++)
		if (ptr[i].type == type)
			for (int k = 0; k < 3; k++) {
				ptr[i].px[k] = ptr[i].x[k] + (sep_rand() - 0.5) * 0.01;
				ptr[i].pv[k] = ptr[i].v[k] + (sep_rand() - 0.5) * 0.01;
			}
}

/* ---- per-type helpers (source/sepmisc.c) ------------------------------------------------ */

int sep_count_type(seppart *ptr, char type, int npart)
{
	int n = 0;
	for (int i = 0; i < npart; i++)
		if (ptr[i].type == type) n++;
	return n;
}

void sep_set_charge(seppart *ptr, char type, double z, sepsys sys)
{
	rt_ctx *c = rt_get(ptr, __func__);
	rt_host_modified(c);
	for (long i = 0; i < sys.npart; i++)
		if (ptr[i].type == type) ptr[i].z = z;
}

void sep_set_mass(seppart *ptr, char type, double m, sepsys sys)
{
	rt_ctx *c = rt_get(ptr, __func__);
	rt_host_modified(c);
	for (long i = 0; i < sys.npart; i++)
		if (ptr[i].type == type) ptr[i].m = m;
}

void sep_set_x0(seppart *ptr, int npart)
{
	rt_ctx *c = rt_get(ptr, __func__);
	rt_need_host(c);
	c->x0_valid = 0;
	for (int i = 0; i < npart; i++)
		for (int k = 0; k < 3; k++) ptr[i].x0[k] = ptr[i].x[k];
}

void sep_set_xn(seppart *ptr, int npart)
{
	rt_ctx *c = rt_get(ptr, __func__);
	rt_host_modified(c);
	for (int i = 0; i < npart; i++)
		for (int k = 0; k < 3; k++) ptr[i].xn[k] = ptr[i].x[k];
}

/* mean momentum per degree of freedom (source/sepmisc.c:576-587); an
 * observation point */
double sep_eval_mom(seppart *ptr, int npart)
{
	rt_ctx *c = rt_get(ptr, __func__);
	rt_need_host(c);
	double mom = 0.0;
	for (int i = 0; i < npart; i++)
		for (int k = 0; k < 3; k++) mom += ptr[i].v[k] * ptr[i].m;
	return mom / (npart * 3);
}

/* xyz writer (source/sepmisc.c:536-574); an observation point */
void sep_save_xyz(seppart *ptr, const char *partnames, const char *file, char *mode, sepsys *sys)
{
	rt_ctx *c = rt_get(ptr, __func__);
	rt_need_host(c);
	FILE *fout = fopen(file, mode);
	if (!fout) sep_error("%s at line %d: I couldn't open file\n", __func__, __LINE__);
	const long ntype = (long)strlen(partnames);
	long ntotal = 0;
	for (long t = 0; t < ntype; t++) ntotal += sep_count_type(ptr, partnames[t], (int)sys->npart);
	fprintf(fout, "%lu\n%f %f %f\n", ntotal, sys->length[0], sys->length[1], sys->length[2]);
	for (long i = 0; i < sys->npart; i++)
		for (long t = 0; t < ntype; t++)
			if (ptr[i].type == partnames[t])
				fprintf(fout, "%c %.15f %.15f %.15f %.15f %.15f %.15f %.15f %.15f\n",
					ptr[i].type, ptr[i].x[0], ptr[i].x[1], ptr[i].x[2], ptr[i].v[0],
					ptr[i].v[1], ptr[i].v[2], ptr[i].m, ptr[i].z);
	fclose(fout);
}

/* ---- resets (source/sepret.c:19-47, source/sepmisc.c:393-431) ------------------------- */

/* sepret handed to the device path are tracked by address; reading one back
 * before zeroing keeps earlier operations in order */
static void flush_ret(sepret *r);

void sep_reset_retval(sepret *r)
{
	flush_ret(r);
	r->epot = 0; r->ecoul = 0; r->ekin = 0; r->sumv2 = 0;
	for (int k = 0; k < 3; k++)
		for (int kk = 0; kk < 3; kk++) {
			r->pot_P[k][kk] = 0.0; r->kin_P[k][kk] = 0.0; r->P[k][kk] = 0.0;
			r->pot_P_conservative[k][kk] = 0.0; r->pot_P_random[k][kk] = 0.0;
			r->pot_P_dissipative[k][kk] = 0.0; r->pot_P_bond[k][kk] = 0.0;
			r->pot_P_mol[k][kk] = 0.0; r->kin_P_mol[k][kk] = 0.0; r->P_mol[k][kk] = 0.0;
			r->pot_T_mol[k][kk] = 0.0; r->kin_T_mol[k][kk] = 0.0; r->T_mol[k][kk] = 0.0;
		}
}

void sep_reset_force(seppart *ptr, sepsys *sys)
{
	rt_ctx *c = rt_get(ptr, __func__);
	sys->max_dist2 = 0.0;
	if (c->dev && c->dev_valid) {
		/* stored device forces become logically zero; pending friction dies with them */
		if (c->pass_slot >= 0) rt_launch_pass(c);
		rt_launch_bonded(c);
		c->forces_zero = 1;
		c->friction = 0;
		c->friction_alpha = 0.0;
		c->host_valid = 0;
	} else {
		for (long i = 0; i < sys->npart; i++)
			for (int k = 0; k < 3; k++) ptr[i].f[k] = 0.0;
	}
}

/* source/sepmisc.c:403-425: zero the molecular forces; the reference
 * exits when sep_init_mol did not enable them.  Here the molecular virial
 * of the passes so far and the per-atom intermolecular forces are zeroed
 * (pending passes run first, so they count in the window they belong to). */
void sep_reset_force_mol(sepsys *sys)
{
	sys->fun_cstate = 0;
	if (sys->molptr->flag_Fij == 0)
		sep_error("%s: Tried to reset mol force, but flag is zero", __func__);
	rt_ctx *c = rt_find_molinfo(sys->molptr);
	if (!c) return;
	if (c->dev) {
		rt_flush(c);
		if (c->mv_uploaded) rt_check(sepdev_molvir_reset(c->dev), "molecular force reset");
	}
	for (int q = 0; q < 9; q++) c->molW[q] = c->molN[q] = 0.0;
}

/* ---- pressure (source/sepret.c:50-82) -------------------------------------------------- */

double sep_get_pressure(sepret *r, sepsys *sys)
{
	sep_pressure_tensor(r, sys);
	return r->p;
}

double sep_get_temperature(sepret *r, sepsys *sys)
{
	flush_ret(r);
	return 2.0 / (3.0 * sys->ndof) * r->ekin;
}

void sep_pressure_tensor(sepret *r, sepsys *sys)
{
	flush_ret(r);
	const double iv = 1.0 / sys->volume;
	for (int k = 0; k < 3; k++)
		for (int kk = 0; kk < 3; kk++) r->P[k][kk] = (r->kin_P[k][kk] + r->pot_P[k][kk]) * iv;
	r->p = (r->P[0][0] + r->P[1][1] + r->P[2][2]) / 3.0;
}

/* flush every context that still has operations recorded for r */
extern rt_ctx *rt_each(int k);
static void flush_ret(sepret *r)
{
	for (int k = 0;; k++) {
		int more = 0;
		rt_ctx *c = rt_each(k);
		if (c == (rt_ctx *)-1) break;
		if (c && rt_ret_pending(c, r)) { rt_flush(c); more = 1; }
		(void)more;
	}
}
