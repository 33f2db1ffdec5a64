/*
 * sep_api_sampler.c - the sacf, vacf, msd, msacf, mvacf and mgh samplers of
 * the sep C API.
 *
 * Control flow, sampling intervals, normalisations and output files follow
 * the reference (source/sepsampler.c:4-242 dispatch, :280-351 sacf,
 * :361-470 radial, :471-641 msd, :658-714 vacf, :725-818 msacf, :822-1105
 * gh, :1110-1410 mgh, :1418-1510 profs, :1531-1666 mprofs, :1757-1825 mvacf,
 * :1828-1916 mavacf, :1918-2051 mmsd,
 * :2055-2213 scatt).  The stress autocorrelations work on the sepret values the host
 * already has (the molecular one through sep_mol_pressure_tensor); vacf,
 * msd, mvacf and mgh keep their particle data on the GPU (dev_sampler.cu,
 * dev_molsampler.cu) and only their per-sample or per-block sums come back
 * to the host.
 */
#include <complex.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "sep.h"
#include "sep_rt.h"

struct sepsacf {
	int lvec, isample, i;
	long nsample;
	double dtsample;
	double *sacf;          /* lvec */
	double *stress;        /* lvec x 3 */
};

struct sepvacf {
	int lvec, isample, i;
	long nsample;
	double dtsample;
	double *vacf;          /* lvec */
	double *block;         /* lvec, scratch */
	sepdev_vacf *dev;
	rt_ctx *ctx;
};

struct sepmsd {
	int lvec, isample, i, nk, logflag;
	long logcounter, nsample, npart;
	char type;
	double *msd, *msdsq, *time, *k;
	double *Fs;            /* lvec x nk (real part) */
	double *out;           /* 2 + nk, scratch */
	sepdev_msd *dev;
	rt_ctx *ctx;
};

/* per-sample Fourier sums of one block and the accumulated correlations;
 * the reference's conjugate sums (fkm) are the complex conjugates of fk for
 * the real weights, and its conjugate auxiliary sum is never used */
struct sepgh {
	int lvec, isample, i, nk;
	long nsample, ncalls;
	double dtsample, avekin;
	double *k;
	double complex *fk_tv, *fk_lv, *fk_rho, *fk_e, *fk_X;
	double complex *c_tv, *c_lv, *c_scatt, *c_e, *c_re, *c_rj, *c_ej, *c_er, *c_jr, *c_je, *c_X;
	double *out;           /* 15 nk, scratch */
	sepdev_gh *dev;
	rt_ctx *ctx;
};

struct sepmmsd {
	int lvec, isample, i, nk, nmol;
	long nsample;
	char type;
	double dtsample;
	double *k, *msd, *Fs;  /* Fs: lvec x nk (real part) */
	double *out;           /* 1 + nk, scratch */
	unsigned char *sel;    /* nmol, scratch */
	sepdev_moltab *tab;
	sepdev_mmsd *dev;
	rt_ctx *ctx;
};

/* all type combinations of one scatt sampler; the program's sepsampler
 * holds a one-element array pointing to it.  intropt 'a': every particle of
 * the types; 'i': the first type from molecules of even index, the second
 * from molecules of odd index or none (sep_set_inter_scatt). */
struct sepscatt {
	int lvec, isample, nk, ntypes, ncomb, index;
	long nsample;
	char types[8], intropt;
	double tspan;
	double complex *p1, *m2;   /* ncomb x lvec x nk */
	double complex *sc;        /* ncomb x lvec x nk */
	double *out;               /* nk x 28, scratch */
};

struct sepmprofs {
	int lvec, isample, dir, dirvel, diramom, nmol;
	long nsample;
	char type;
	double *acc;           /* lvec x 16 accumulated sums */
	double *out;           /* lvec x 16, scratch */
	unsigned char *sel;    /* nmol, scratch */
	sepdev_moltab *tab;
	rt_ctx *ctx;
};

struct sepradial {
	int lvec, isample, ntypes, ncomb;
	long nsample;
	char types[8];
	double *hist;          /* lvec x ncomb accumulated counts */
	double *out;           /* lvec x ncomb, scratch */
	unsigned *mask;        /* [SEPDEV_MAXTYPES]^2, scratch */
};

struct sepprofs {
	int lvec, isample, dir, dirvel;
	long nsample;
	char type;
	double *momc, *svel, *dens, *temp;   /* lvec each */
	double *hist;                        /* 4 lvec, scratch */
};

struct sepmsacf {
	int lvec, isample, i;
	long nsample;
	double dtsample;
	double *sacf;          /* lvec x 2: symmetric, antisymmetric */
	double *sstress;       /* lvec x 3 */
	double *astress;       /* lvec x 3 */
};

/* mavacf keeps the same window as mvacf (its own quantity per molecule) */
struct sepmavacf {
	int lvec, isample, i;
	long nsample;
	double dtsample;
	double *vacf, *block;
	unsigned char *sel;
	sepdev_vacf *dev;
	sepdev_moltab *tab;
	rt_ctx *ctx;
};

struct sepmvacf {
	int lvec, isample, i;
	long nsample;
	double dtsample;
	double *vacf;          /* lvec */
	double *block;         /* lvec, scratch */
	sepdev_vacf *dev;
	sepdev_moltab *tab;
	rt_ctx *ctx;
};

/* the per-sample Fourier sums of one block (fk) and the accumulated
 * correlations (c); the conjugate sums the reference also keeps (fkm) are
 * the complex conjugates of these */
struct sepmgh {
	int lvec, isample, i, nk, safe;
	long nsample, ncalls;
	double dtsample, avekin;
	double *k;
	double complex *fk_tv, *fk_lv, *fk_rho, *fk_tav, *fk_lav, *fk_e, *fk_dip, *fk_X;
	double complex *c_tv, *c_lv, *c_scatt, *c_tav, *c_lav, *c_e, *c_vav, *c_dip, *c_X;
	double *out;           /* 18 nk + 1, scratch */
	sepdev_moltab *tab;
	rt_ctx *ctx;
};

static void *xcalloc(size_t n, size_t s)
{
	void *p = calloc(n ? n : 1, s);
	if (!p) sep_error("couldn't allocate memory");
	return p;
}

sepsampler sep_init_sampler(void)
{
	sepsampler a;
	memset(&a, 0, sizeof a);
	return a;
}

void sep_add_mol_sampler(sepsampler *sptr, sepmol *mols)
{
	sptr->molptr = mols;
}

static int sample_interval(double tsample, int lvec, double dt, double *dtsample)
{
	*dtsample = tsample / lvec;
	const int is = (int)(*dtsample / dt);
	if (is < 1) sep_error("%s: isample is too small - CHECK lvec argument", __func__);
	return is;
}

void sep_add_sampler(sepsampler *sptr, const char *sampler, sepsys sys, int lvec, ...)
{
	va_list args;
	va_start(args, lvec);
	if (strcmp(sampler, "sacf") == 0) {
		if (sptr->flag_sacf != 1) {
			const double tsample = va_arg(args, double);
			struct sepsacf *p = xcalloc(1, sizeof *p);
			p->lvec = lvec;
			p->isample = sample_interval(tsample, lvec, sys.dt, &p->dtsample);
			p->sacf = xcalloc(lvec, sizeof(double));
			p->stress = xcalloc(3 * (size_t)lvec, sizeof(double));
			sptr->sacf = p;
			sptr->flag_sacf = 1;
		}
	} else if (strcmp(sampler, "vacf") == 0) {
		if (sptr->flag_vacf != 1) {
			const double tsample = va_arg(args, double);
			struct sepvacf *p = xcalloc(1, sizeof *p);
			p->lvec = lvec;
			p->isample = sample_interval(tsample, lvec, sys.dt, &p->dtsample);
			p->vacf = xcalloc(lvec, sizeof(double));
			p->block = xcalloc(lvec, sizeof(double));
			sptr->vacf = p;
			sptr->flag_vacf = 1;
		}
	} else if (strcmp(sampler, "msd") == 0) {
		if (sptr->flag_msd != 1) {
			const double tsample = va_arg(args, double);
			const int nk = va_arg(args, int);
			const char type = (char)va_arg(args, int);
			struct sepmsd *p = xcalloc(1, sizeof *p);
			p->nk = nk;
			p->type = type;
			p->npart = (long)sys.npart;
			if (lvec > 0) {
				p->lvec = lvec;
				p->isample = sample_interval(tsample, lvec, sys.dt, &(double){0.0});
				const double dts = tsample / lvec;
				p->time = xcalloc(lvec, sizeof(double));
				for (int n = 0; n < lvec; n++) p->time[n] = dts * (n + 1);
			} else {
				/* log-spaced: dt, 2 dt, 4 dt, ... up to tsample */
				double t = sys.dt;
				lvec = 1;
				while (t < tsample) { lvec++; t = 2 * t; }
				p->lvec = lvec;
				p->logflag = 1;
				p->time = xcalloc(lvec, sizeof(double));
				long m = 1;
				for (int c = 0; c < lvec; c++) { p->time[c] = sys.dt * m; m = 2 * m; }
				p->logcounter = 1;
			}
			p->msd = xcalloc(p->lvec, sizeof(double));
			p->msdsq = xcalloc(p->lvec, sizeof(double));
			p->Fs = xcalloc((size_t)p->lvec * (nk > 0 ? nk : 1), sizeof(double));
			p->k = xcalloc(nk, sizeof(double));
			p->out = xcalloc(2 + nk, sizeof(double));
			FILE *f = fopen("msd-k.dat", "w");
			if (!f) sep_error("%s: couldn't open file", __func__);
			for (int n = 1; n <= nk; n++) {
				p->k[n - 1] = 2 * SEP_PI / sys.length[0] * n;
				fprintf(f, "%f\n", p->k[n - 1]);
			}
			fclose(f);
			sptr->msd = p;
			sptr->flag_msd = 1;
		}
	} else if (strcmp(sampler, "msacf") == 0) {
		if (sptr->flag_msacf != 1) {
			if (sptr->molptr == NULL) sep_error("%s: molpointer not initialized", __func__);
			const double tsample = va_arg(args, double);
			struct sepmsacf *p = xcalloc(1, sizeof *p);
			p->lvec = lvec;
			p->isample = sample_interval(tsample, lvec, sys.dt, &p->dtsample);
			p->sacf = xcalloc(2 * (size_t)lvec, sizeof(double));
			p->sstress = xcalloc(3 * (size_t)lvec, sizeof(double));
			p->astress = xcalloc(3 * (size_t)lvec, sizeof(double));
			sptr->msacf = p;
			sptr->flag_msacf = 1;
		}
	} else if (strcmp(sampler, "mgh") == 0) {
		if (sptr->flag_mgh != 1) {
			if (sptr->molptr == NULL) sep_error("%s: molpointer not initialized", __func__);
			const double tsample = va_arg(args, double);
			const int nk = va_arg(args, int);
			const int safe = va_arg(args, int);
			struct sepmgh *p = xcalloc(1, sizeof *p);
			p->lvec = lvec;
			p->isample = sample_interval(tsample, lvec, sys.dt, &p->dtsample);
			p->nk = nk;
			p->k = xcalloc(nk, sizeof(double));
			FILE *f = fopen("mgh-wavevector.dat", "w");
			if (!f) sep_error("%s: couldn't open file", __func__);
			for (int n = 1; n <= nk; n++) {
				p->k[n - 1] = 2 * SEP_PI * n / sys.length[1];
				fprintf(f, "%f\n", p->k[n - 1]);
			}
			fclose(f);
			p->safe = safe ? 1 : 0;
			if (!p->safe)
				sep_warning("ACHTUNG - unsafe mode for mgh sampler. Assuming uniaxial single component system");
			const size_t m = (size_t)lvec * (nk > 0 ? nk : 1);
			double complex **arr[] = {&p->fk_tv, &p->fk_lv, &p->fk_rho, &p->fk_tav, &p->fk_lav, &p->fk_e,
						  &p->fk_dip, &p->fk_X, &p->c_tv, &p->c_lv, &p->c_scatt, &p->c_tav,
						  &p->c_lav, &p->c_e, &p->c_vav, &p->c_dip, &p->c_X};
			for (size_t q = 0; q < sizeof arr / sizeof arr[0]; q++) *arr[q] = xcalloc(m, sizeof(double complex));
			p->out = xcalloc(18 * (size_t)nk + 1, sizeof(double));
			sptr->mgh = p;
			sptr->flag_mgh = 1;
		}
	} else if (strcmp(sampler, "profs") == 0) {
		if (sptr->flag_profs != 1) {
			const char type = (char)va_arg(args, int);
			const int isample = va_arg(args, int);
			struct sepprofs *p = xcalloc(1, sizeof *p);
			p->lvec = lvec;
			p->isample = isample;
			p->type = type;
			/* the reference's defaults: profiles along z of v_x */
			p->dir = 2;
			p->dirvel = 0;
			p->momc = xcalloc(lvec, sizeof(double));
			p->svel = xcalloc(lvec, sizeof(double));
			p->dens = xcalloc(lvec, sizeof(double));
			p->temp = xcalloc(lvec, sizeof(double));
			p->hist = xcalloc(4 * (size_t)lvec, sizeof(double));
			sptr->profs = p;
			sptr->flag_profs = 1;
		}
	} else if (strcmp(sampler, "gh") == 0) {
		if (sptr->flag_gh != 1) {
			const double tsample = va_arg(args, double);
			const int nk = va_arg(args, int);
			struct sepgh *p = xcalloc(1, sizeof *p);
			p->lvec = lvec;
			p->isample = sample_interval(tsample, lvec, sys.dt, &p->dtsample);
			p->nk = nk;
			p->k = xcalloc(nk, sizeof(double));
			FILE *f = fopen("gh-wavevector.dat", "w");
			if (!f) sep_error("%s: couldn't open file", __func__);
			for (int n = 1; n <= nk; n++) {
				p->k[n - 1] = 2 * SEP_PI * n / sys.length[1];
				fprintf(f, "%f\n", p->k[n - 1]);
			}
			fclose(f);
			const size_t m = (size_t)lvec * (nk > 0 ? nk : 1);
			double complex **arr[] = {&p->fk_tv, &p->fk_lv, &p->fk_rho, &p->fk_e, &p->fk_X, &p->c_tv, &p->c_lv,
						  &p->c_scatt, &p->c_e, &p->c_re, &p->c_rj, &p->c_ej, &p->c_er, &p->c_jr,
						  &p->c_je, &p->c_X};
			for (size_t q = 0; q < sizeof arr / sizeof arr[0]; q++) *arr[q] = xcalloc(m, sizeof(double complex));
			p->out = xcalloc(15 * (size_t)(nk > 0 ? nk : 1), sizeof(double));
			sptr->gh = p;
			sptr->flag_gh = 1;
		}
	} else if (strcmp(sampler, "radial") == 0) {
		if (sptr->flag_radial != 1) {
			const int isample = va_arg(args, int);
			const char *t = va_arg(args, char *);
			struct sepradial *p = xcalloc(1, sizeof *p);
			p->lvec = lvec;
			p->isample = isample;
			p->ntypes = (int)strlen(t);
			if (p->ntypes < 1 || p->ntypes > 7)
				sep_error("%s: radial takes 1 to 7 types (got \"%s\")", __func__, t);
			memcpy(p->types, t, p->ntypes);
			for (int k = 1; k <= p->ntypes; k++) p->ncomb += k;
			p->hist = xcalloc((size_t)lvec * p->ncomb, sizeof(double));
			p->out = xcalloc((size_t)lvec * p->ncomb, sizeof(double));
			p->mask = xcalloc(SEPDEV_MAXTYPES * SEPDEV_MAXTYPES, sizeof(unsigned));
			FILE *f = fopen("radial_info.dat", "w");
			if (!f) sep_error("%s: Couldn't open file", __func__);
			fprintf(f, "Pairs in radial.dat columns are\n");
			for (int a = 0; a < p->ntypes; a++)
				for (int b = a; b < p->ntypes; b++) fprintf(f, "%c%c  ", p->types[a], p->types[b]);
			fclose(f);
			sptr->radial = p;
			sptr->flag_radial = 1;
		}
	} else if (strcmp(sampler, "mmsd") == 0) {
		if (sptr->flag_mmsd != 1) {
			const double tsample = va_arg(args, double);
			const int nk = va_arg(args, int);
			const char type = (char)va_arg(args, int);
			struct sepmmsd *p = xcalloc(1, sizeof *p);
			p->lvec = lvec;
			p->isample = sample_interval(tsample, lvec, sys.dt, &p->dtsample);
			p->nk = nk;
			p->type = type;
			p->nmol = (int)sys.molptr->num_mols;
			p->k = xcalloc(nk, sizeof(double));
			FILE *f = fopen("mmsd-wavevector.dat", "w");
			if (!f) sep_error("%s: Couldn't open file", __func__);
			for (int n = 1; n <= nk; n++) {
				p->k[n - 1] = 2 * SEP_PI / sys.length[0] * n;
				fprintf(f, "%f\n", p->k[n - 1]);
			}
			fclose(f);
			p->msd = xcalloc(lvec, sizeof(double));
			p->Fs = xcalloc((size_t)lvec * (nk > 0 ? nk : 1), sizeof(double));
			p->out = xcalloc(1 + nk, sizeof(double));
			p->sel = xcalloc(p->nmol, 1);
			sptr->mmsd = p;
			sptr->flag_mmsd = 1;
		}
	} else if (strcmp(sampler, "scatt") == 0) {
		if (sptr->flag_scatt != 1) {
			const char *t = va_arg(args, char *);
			const int nk = va_arg(args, int);
			const double tsample = va_arg(args, double);
			struct sepscatt *p = xcalloc(1, sizeof *p);
			p->ntypes = (int)strlen(t);
			if (p->ntypes < 1 || p->ntypes > 7)
				sep_error("%s: scatt takes 1 to 7 types (got \"%s\")", __func__, t);
			memcpy(p->types, t, p->ntypes);
			p->ncomb = p->ntypes * (p->ntypes + 1) / 2;
			p->lvec = lvec;
			p->nk = nk;
			p->tspan = tsample;
			p->isample = (int)(tsample / (lvec * sys.dt));
			if (p->isample < 1) sep_error("%s: isample is too small - CHECK lvec argument", __func__);
			p->intropt = 'a';
			const size_t m = (size_t)p->ncomb * lvec * (nk > 0 ? nk : 1);
			p->p1 = xcalloc(m, sizeof(double complex));
			p->m2 = xcalloc(m, sizeof(double complex));
			p->sc = xcalloc(m, sizeof(double complex));
			p->out = xcalloc(28 * (size_t)(nk > 0 ? nk : 1), sizeof(double));
			sptr->scatt = xcalloc(1, sizeof(struct sepscatt *));
			sptr->scatt[0] = p;
			sptr->flag_scatt = 1;
		}
	} else if (strcmp(sampler, "mprofs") == 0) {
		if (sptr->flag_mprofs != 1) {
			const char type = (char)va_arg(args, int);
			const int isample = va_arg(args, int);
			struct sepmprofs *p = xcalloc(1, sizeof *p);
			p->lvec = lvec;
			p->isample = isample;
			p->type = type;
			/* the reference's fixed choice: profiles along z of v_x, the
			 * angular velocity's y component */
			p->dir = 2;
			p->dirvel = 0;
			p->diramom = 1;
			p->nmol = (int)sys.molptr->num_mols;
			p->acc = xcalloc(16 * (size_t)lvec, sizeof(double));
			p->out = xcalloc(16 * (size_t)lvec, sizeof(double));
			p->sel = xcalloc(p->nmol > 0 ? p->nmol : 1, 1);
			sptr->mprofs = p;
			sptr->flag_mprofs = 1;
		}
	} else if (strcmp(sampler, "mavacf") == 0) {
		if (sptr->flag_mavacf != 1) {
			const double tsample = va_arg(args, double);
			struct sepmavacf *p = xcalloc(1, sizeof *p);
			p->lvec = lvec;
			p->isample = sample_interval(tsample, lvec, sys.dt, &p->dtsample);
			p->vacf = xcalloc(lvec, sizeof(double));
			p->block = xcalloc(lvec, sizeof(double));
			p->sel = xcalloc(sys.molptr->num_mols > 0 ? sys.molptr->num_mols : 1, 1);
			sptr->mavacf = p;
			sptr->flag_mavacf = 1;
		}
	} else if (strcmp(sampler, "mvacf") == 0) {
		if (sptr->flag_mvacf != 1) {
			const double tsample = va_arg(args, double);
			struct sepmvacf *p = xcalloc(1, sizeof *p);
			p->lvec = lvec;
			p->isample = sample_interval(tsample, lvec, sys.dt, &p->dtsample);
			p->vacf = xcalloc(lvec, sizeof(double));
			p->block = xcalloc(lvec, sizeof(double));
			sptr->mvacf = p;
			sptr->flag_mvacf = 1;
		}
	} else {
		va_end(args);
		sep_error("%s: sampler %s is not provided by this GPU implementation "
			  "(available: sacf, vacf, msd, msacf, mvacf, mavacf, gh, mgh, profs, mprofs, radial, mmsd, scatt)",
			  __func__,
			  sampler);
	}
	va_end(args);
}

/* ---- sacf: source/sepsampler.c:305-348 ---- */
static void sacf_sample(struct sepsacf *s, sepret *ret, sepsys sys)
{
	sep_pressure_tensor(ret, &sys);
	const int i = s->i;
	s->stress[3 * i] = -ret->P[0][1];
	s->stress[3 * i + 1] = -ret->P[0][2];
	s->stress[3 * i + 2] = -ret->P[1][2];
	s->i++;
	if (s->i == s->lvec) {
		for (int n = 0; n < s->lvec; n++) {
			double acc = 0.0;
			for (int k = 0; k < 3; k++)
				for (int m = 0; m < s->lvec - n; m++) acc += s->stress[3 * m + k] * s->stress[3 * (n + m) + k];
			s->sacf[n] += acc;
		}
		s->nsample++;
		FILE *f = fopen("sacf.dat", "w");
		if (!f) sep_error("%s: couldn't open file", __func__);
		for (int n = 0; n < s->lvec; n++) {
			const double t = n * s->dtsample;
			const double fac = sys.volume / (3.0 * (s->lvec - n) * s->nsample);
			fprintf(f, "%f %f\n", t, s->sacf[n] * fac);
		}
		fclose(f);
		s->i = 0;
	}
}

static rt_ctx *sampler_ctx(seppart *pptr, sepsys *sys)
{
	rt_ctx *c = rt_get(pptr, "sep_sample");
	rt_need_device(c, sys);
	return c;
}

/* ---- vacf: source/sepsampler.c:683-711 ---- */
static void vacf_sample(struct sepvacf *s, seppart *pptr, sepsys sys)
{
	rt_ctx *c = sampler_ctx(pptr, &sys);
	if (!s->dev || s->ctx != c) {
		if (s->dev) sepdev_vacf_destroy(s->dev);
		rt_check(sepdev_vacf_create(c->dev, s->lvec, &s->dev), "vacf sampler");
		s->ctx = c;
	}
	rt_check(sepdev_vacf_store(c->dev, s->dev, s->i), "vacf sample");
	s->i++;
	if (s->i == s->lvec) {
		rt_check(sepdev_vacf_block(c->dev, s->dev, s->block), "vacf block");
		for (int k = 0; k < s->lvec; k++) s->vacf[k] += s->block[k];
		s->nsample++;
		FILE *f = fopen("vacf.dat", "w");
		if (!f) sep_error("%s: couldn't open file", __func__);
		for (int k = 0; k < s->lvec; k++) {
			const double t = k * s->dtsample;
			const double fac = 1.0 / ((double)(s->lvec - k) * sys.npart * s->nsample);
			fprintf(f, "%f %f\n", t, s->vacf[k] * fac);
		}
		fclose(f);
		s->i = 0;
	}
}

/* ---- msd: source/sepsampler.c:554-638 ---- */
static void msd_sample(struct sepmsd *s, seppart *pptr, sepsys sys)
{
	rt_ctx *c = sampler_ctx(pptr, &sys);
	if (!s->dev || s->ctx != c) {
		if (s->dev) sepdev_msd_destroy(s->dev);
		rt_check(sepdev_msd_create(c->dev, s->nk, s->k, &s->dev), "msd sampler");
		s->ctx = c;
	}
	int index = s->i;
	if (index == 0) rt_check(sepdev_msd_base(c->dev, s->dev), "msd reference positions");
	int tid = -1;
	for (int t = 0; t < c->ntypes; t++)
		if (c->tchar[t] == s->type) tid = t;
	rt_check(sepdev_msd_sample(c->dev, s->dev, tid, s->out), "msd sample");
	s->msd[index] += s->out[0];
	s->msdsq[index] += s->out[1];
	for (int j = 0; j < s->nk; j++) s->Fs[(size_t)index * s->nk + j] += s->out[2 + j];
	index++;
	if (index == s->lvec) {
		s->nsample++;
		const int ntype = sep_count_type(pptr, s->type, (int)s->npart);
		FILE *f = fopen("msd.dat", "w");
		if (!f) sep_error("%s: couldn't open file", __func__);
		for (int n = 0; n < s->lvec; n++) fprintf(f, "%f %f \n", s->time[n], s->msd[n] / (ntype * s->nsample));
		fclose(f);
		f = fopen("msd-gaussparam.dat", "w");
		if (!f) sep_error("%s: couldn't open file", __func__);
		for (int n = 0; n < s->lvec; n++) {
			const double a = s->msdsq[n] / (ntype * s->nsample);
			const double m = s->msd[n] / (ntype * s->nsample);
			fprintf(f, "%f %f \n", s->time[n], 3.0 * a / (5.0 * m * m) - 1.);
		}
		fclose(f);
		f = fopen("msd-incoherent.dat", "w");
		if (!f) sep_error("%s: couldn't open file", __func__);
		for (int n = 0; n < s->lvec; n++) {
			fprintf(f, "%f ", s->time[n]);
			for (int j = 0; j < s->nk; j++) fprintf(f, "%f ", s->Fs[(size_t)n * s->nk + j] / (s->nsample * ntype));
			fprintf(f, "\n");
		}
		fclose(f);
		index = 0;
	}
	s->i = index;
}

/* ---- msacf: source/sepsampler.c:752-808 ---- */
static void msacf_sample(struct sepmsacf *s, seppart *pptr, sepmol *mols, sepret *ret, sepsys sys)
{
	sep_mol_pressure_tensor(pptr, mols, ret, &sys);
	const int i = s->i;
	s->sstress[3 * i] = 0.5 * (ret->P_mol[0][1] + ret->P_mol[1][0]);
	s->sstress[3 * i + 1] = 0.5 * (ret->P_mol[0][2] + ret->P_mol[2][0]);
	s->sstress[3 * i + 2] = 0.5 * (ret->P_mol[1][2] + ret->P_mol[2][1]);
	s->astress[3 * i] = 0.5 * (ret->P_mol[0][1] - ret->P_mol[1][0]);
	s->astress[3 * i + 1] = 0.5 * (ret->P_mol[0][2] - ret->P_mol[2][0]);
	s->astress[3 * i + 2] = 0.5 * (ret->P_mol[1][2] - ret->P_mol[2][1]);
	s->i++;
	if (s->i == s->lvec) {
		for (int n = 0; n < s->lvec; n++) {
			double as = 0.0, aa = 0.0;
			for (int k = 0; k < 3; k++)
				for (int m = 0; m < s->lvec - n; m++) {
					as += s->sstress[3 * m + k] * s->sstress[3 * (n + m) + k];
					aa += s->astress[3 * m + k] * s->astress[3 * (n + m) + k];
				}
			s->sacf[2 * n] += as;
			s->sacf[2 * n + 1] += aa;
		}
		s->nsample++;
		FILE *f = fopen("msacf.dat", "w");
		if (!f) sep_error("%s: couldn't open file", __func__);
		for (int n = 0; n < s->lvec; n++) {
			const double t = n * s->dtsample;
			const double fac = sys.volume / (3.0 * (s->lvec - n) * s->nsample);
			fprintf(f, "%f %f %f\n", t, s->sacf[2 * n] * fac, s->sacf[2 * n + 1] * fac);
		}
		fclose(f);
		s->i = 0;
	}
}

/* the molecule tables of the sampler's molecules on the context's device */
static void mol_tables(sepdev_moltab **tab, rt_ctx **owner, rt_ctx *c, sepmol *mols, sepsys *sys)
{
	if (*tab && *owner == c) return;
	if (*tab) sepdev_moltab_destroy(*tab);
	*tab = NULL;
	if (mols == NULL) sep_error("sep_sample: molpointer not initialized");
	const int nm = (int)sys->molptr->num_mols;
	int *first = xcalloc(nm, sizeof(int)), *nuau = xcalloc(nm, sizeof(int));
	int *start = xcalloc(nm + 1, sizeof(int));
	double *mass = xcalloc(nm, sizeof(double));
	for (int m = 0; m < nm; m++) start[m + 1] = start[m] + (int)mols[m].nuau;
	int *atoms = xcalloc(start[nm], sizeof(int));
	for (int m = 0; m < nm; m++) {
		first[m] = mols[m].nuau > 0 ? mols[m].index[0] : 0;
		nuau[m] = (int)mols[m].nuau;
		mass[m] = mols[m].m;
		for (unsigned q = 0; q < mols[m].nuau; q++) atoms[start[m] + q] = mols[m].index[q];
	}
	rt_check(sepdev_moltab_create(c->dev, nm, first, nuau, start, atoms, mass, tab), "molecule tables");
	*owner = c;
	free(first); free(nuau); free(start); free(atoms); free(mass);
}

/* ---- mvacf: source/sepsampler.c:1782-1816 ---- */
static void mvacf_sample(struct sepmvacf *s, seppart *pptr, sepmol *mols, sepsys sys)
{
	rt_ctx *c = sampler_ctx(pptr, &sys);
	const int nm = (int)sys.molptr->num_mols;
	if (s->ctx != c) {
		if (s->dev) sepdev_vacf_destroy(s->dev);
		s->dev = NULL;
	}
	mol_tables(&s->tab, &s->ctx, c, mols, &sys);
	if (!s->dev) rt_check(sepdev_vacf_create_count(c->dev, s->lvec, nm, &s->dev), "mvacf sampler");
	rt_check(sepdev_mvacf_store(c->dev, s->tab, s->dev, s->i), "mvacf sample");
	s->i++;
	if (s->i == s->lvec) {
		rt_check(sepdev_vacf_block(c->dev, s->dev, s->block), "mvacf block");
		for (int k = 0; k < s->lvec; k++) s->vacf[k] += s->block[k];
		s->nsample++;
		FILE *f = fopen("mvacf.dat", "w");
		if (!f) sep_error("%s: couldn't open file", __func__);
		for (int k = 0; k < s->lvec; k++) {
			const double t = k * s->dtsample;
			const double fac = 1.0 / ((double)(s->lvec - k) * nm * s->nsample);
			fprintf(f, "%f %f\n", t, s->vacf[k] * fac);
		}
		fclose(f);
		s->i = 0;
	}
}

/* ---- mavacf: source/sepsampler.c:1853-1906 ----
 * The reference's body samples, per molecule, the y component of the
 * end-to-end vector of the type-A molecules times the first particle's
 * |charge| times the molecule mass (its angular-velocity variant is
 * commented out); the block correlation and file follow mvacf's with the
 * times at (k + 1/2) dt_sample. */
static void mavacf_sample(struct sepmavacf *s, seppart *pptr, sepmol *mols, sepsys sys)
{
	rt_ctx *c = sampler_ctx(pptr, &sys);
	const int nm = (int)sys.molptr->num_mols;
	if (nm < 1 || mols == NULL) sep_error("%s: no molecules to sample", __func__);
	if (s->ctx != c) {
		if (s->dev) sepdev_vacf_destroy(s->dev);
		s->dev = NULL;
	}
	mol_tables(&s->tab, &s->ctx, c, mols, &sys);
	if (!s->dev) rt_check(sepdev_vacf_create_count(c->dev, s->lvec, nm, &s->dev), "mavacf sampler");
	for (int i = 0; i < nm; i++) s->sel[i] = mols[i].type == 'A';
	/* charges live on the host; the device never changes them */
	const double q = fabs(pptr[0].z);
	rt_check(sepdev_mavacf_store(c->dev, s->tab, s->dev, s->i, s->sel, (int)mols[0].nuau - 1, q), "mavacf sample");
	s->i++;
	if (s->i == s->lvec) {
		rt_check(sepdev_vacf_block(c->dev, s->dev, s->block), "mavacf block");
		for (int k = 0; k < s->lvec; k++) s->vacf[k] += s->block[k];
		s->nsample++;
		FILE *f = fopen("mavacf.dat", "w");
		if (!f) sep_error("%s: couldn't open file", __func__);
		for (int k = 0; k < s->lvec; k++) {
			const double t = (k + 0.5) * s->dtsample;
			const double fac = 1.0 / ((double)(s->lvec - k) * nm * s->nsample);
			fprintf(f, "%f %f\n", t, s->vacf[k] * fac);
		}
		fclose(f);
		s->i = 0;
	}
}

/* ---- mgh: source/sepsampler.c:1231-1410 ----
 * The reference resets every per-sample sum at the start of a sample except
 * the energy's, which therefore accumulates over the blocks at each index;
 * the running mean kinetic energy starts at 0 here (the reference leaves it
 * unset). */
static void mgh_files(struct sepmgh *g, double volume)
{
	static const char *names[9] = {"mgh-trans-momentum-acf.dat", "mgh-long-momentum-acf.dat",
				       "mgh-rho-acf.dat", "mgh-trans-angmomentum-acf.dat",
				       "mgh-long-angmomentum-acf.dat", "mgh-energy-acf.dat",
				       "mgh-momentum-angmomentum-ccf.dat", "mgh-dipole-acf.dat", "mgh-X-cf.dat"};
	double complex *cs[9] = {g->c_tv, g->c_lv, g->c_scatt, g->c_tav, g->c_lav, g->c_e, g->c_vav, g->c_dip, g->c_X};
	for (int f = 0; f < 9; f++) {
		FILE *fp = fopen(names[f], "w");
		if (!fp) sep_error("%s: Error opening files", __func__);
		if (f == 8 && g->safe) { fclose(fp); continue; }
		for (int n = 0; n < g->lvec; n++) {
			fprintf(fp, "%f ", n * g->dtsample);
			const double fac = 1.0 / (g->nsample * volume * (g->lvec - n));
			for (int k = 0; k < g->nk; k++) {
				const double complex v = cs[f][(size_t)n * g->nk + k] * fac;
				fprintf(fp, "%f %f ", creal(v), cimag(v));
			}
			fprintf(fp, "\n");
		}
		fclose(fp);
	}
}

static void mgh_sample(struct sepmgh *g, seppart *pptr, sepmol *mols, sepsys sys)
{
	rt_ctx *c = sampler_ctx(pptr, &sys);
	mol_tables(&g->tab, &g->ctx, c, mols, &sys);
	rt_check(sepdev_mgh_sample(c->dev, g->tab, g->nk, g->k, !g->safe, g->out), "mgh sample");
	const int nm = (int)sys.molptr->num_mols, nk = g->nk;
	g->ncalls++;
	g->avekin += g->out[18 * nk] / ((double)nm * g->ncalls);
	const size_t row = (size_t)g->i * nk;
	for (int j = 0; j < nk; j++) {
		const double *o = g->out + 18 * j;
		double complex S[9];
		for (int q = 0; q < 9; q++) S[q] = o[2 * q] + I * o[2 * q + 1];
		g->fk_rho[row + j] = S[0];
		g->fk_tv[row + j] = S[1];
		g->fk_lv[row + j] = S[2];
		g->fk_e[row + j] += S[3] - g->avekin * S[4];
		g->fk_tav[row + j] = S[5];
		g->fk_lav[row + j] = S[6];
		g->fk_dip[row + j] = S[7];
		g->fk_X[row + j] = g->safe ? 0.0 : S[8];
	}
	g->i++;
	if (g->i == g->lvec) {
		const int lv = g->lvec;
		for (int k = 0; k < nk; k++)
			for (int n = 0; n < lv; n++) {
				const size_t o = (size_t)n * nk + k;
				for (int m = 0; m < lv - n; m++) {
					const size_t a = (size_t)m * nk + k, b = (size_t)(n + m) * nk + k;
					g->c_tv[o] += conj(g->fk_tv[a]) * g->fk_tv[b];
					g->c_lv[o] += conj(g->fk_lv[a]) * g->fk_lv[b];
					g->c_scatt[o] += g->fk_rho[a] * conj(g->fk_rho[b]);
					g->c_e[o] += g->fk_e[a] * conj(g->fk_e[b]);
					g->c_tav[o] += conj(g->fk_tav[a]) * g->fk_tav[b];
					g->c_lav[o] += conj(g->fk_lav[a]) * g->fk_lav[b];
					/* the reference's vav pair: sums of s_z and of M v_x */
					g->c_vav[o] += conj(g->fk_tv[a]) * g->fk_tav[b];
					g->c_dip[o] += conj(g->fk_dip[a]) * g->fk_dip[b];
					if (!g->safe) g->c_X[o] += conj(g->fk_X[a]) * g->fk_X[b];
				}
			}
		g->nsample++;
		mgh_files(g, sys.volume);
		g->i = 0;
	}
}

/* ---- profs: source/sepsampler.c:1453-1510 ----
 * The bin of a particle is floor(x_dir / dl), the last bin for a coordinate
 * that rounds to L_dir. */
static void profs_sample(struct sepprofs *p, seppart *pptr, sepsys sys)
{
	rt_ctx *c = sampler_ctx(pptr, &sys);
	const int lv = p->lvec, dir = p->dir;
	const double dl = sys.length[dir] / lv;
	double dV;
	if (dir == 0) dV = dl * sys.length[1] * sys.length[2];
	else if (dir == 1) dV = sys.length[0] * dl * sys.length[2];
	else dV = sys.length[0] * sys.length[1] * dl;
	const int tid = rt_type_id(c, p->type);
	for (int k = 0; k < 4 * lv; k++) p->hist[k] = 0.0;
	if (tid >= 0) rt_check(sepdev_profile(c->dev, tid, dir, p->dirvel, lv, p->hist), "profile");
	p->nsample++;
	const double idV = 1.0 / dV;
	for (int n = 0; n < lv; n++) {
		p->momc[n] += p->hist[4 * n] * idV;
		p->dens[n] += p->hist[4 * n + 1] * idV;
		if (p->hist[4 * n + 3] > 0) p->temp[n] += p->hist[4 * n + 2];
	}
	if (p->nsample % 100 == 0) {
		FILE *f = fopen("profs.dat", "w");
		if (!f) sep_error("%s: Couldn't open file", __func__);
		for (int n = 0; n < lv; n++) {
			const double insample = 1.0 / p->nsample;
			double temp_fac = 0;
			if (p->dens[n] > 0.0) {
				p->svel[n] = p->momc[n] / p->dens[n];
				temp_fac = 1.0 / (2.0 * dV * p->dens[n]);
			}
			const double z = (n + 0.5) * dl;
			fprintf(f, "%f %f %f %f %f\n", z, p->momc[n] * insample, p->dens[n] * insample,
				p->temp[n] * temp_fac, p->svel[n]);
		}
		fclose(f);
	}
}

/* ---- gh: source/sepsampler.c:957-1105 ---- */
static void gh_sample(struct sepgh *g, seppart *pptr, sepsys sys)
{
	rt_ctx *c = sampler_ctx(pptr, &sys);
	if (!g->dev || g->ctx != c) {
		if (g->dev) sepdev_gh_destroy(g->dev);
		rt_check(sepdev_gh_create(c->dev, g->nk, g->k, &g->dev), "gh sampler");
		g->ctx = c;
	}
	/* the accelerations are those of the last integrator step: the stored
	 * forces, which calls deferred since then have not touched */
	rt_check(sepdev_gh_sample(c->dev, g->dev, g->out), "gh sample");
	const int nk = g->nk;
	g->ncalls++;
	g->avekin += g->out[14] / ((double)sys.npart * g->ncalls);
	const size_t row = (size_t)g->i * nk;
	for (int j = 0; j < nk; j++) {
		const double *o = g->out + 15 * j;
		double complex S[7];
		for (int q = 0; q < 7; q++) S[q] = o[2 * q] + I * o[2 * q + 1];
		g->fk_rho[row + j] = S[0];
		g->fk_tv[row + j] = S[1];
		g->fk_lv[row + j] = S[2];
		g->fk_e[row + j] = S[3] - g->avekin * S[4];
		g->fk_X[row + j] = S[5] - I * g->k[j] * S[6];
	}
	g->i++;
	if (g->i < g->lvec) return;
	const int lv = g->lvec;
	for (int k = 0; k < nk; k++)
		for (int n = 0; n < lv; n++) {
			const size_t o = (size_t)n * nk + k;
			for (int m = 0; m < lv - n; m++) {
				const size_t a = (size_t)m * nk + k, b = (size_t)(n + m) * nk + k;
				g->c_tv[o] += conj(g->fk_tv[a]) * g->fk_tv[b];
				g->c_lv[o] += conj(g->fk_lv[a]) * g->fk_lv[b];
				g->c_scatt[o] += g->fk_rho[a] * conj(g->fk_rho[b]);
				g->c_e[o] += g->fk_e[a] * conj(g->fk_e[b]);
				g->c_re[o] += g->fk_rho[a] * conj(g->fk_e[b]);
				g->c_rj[o] += g->fk_rho[a] * conj(g->fk_lv[b]);
				g->c_ej[o] += g->fk_e[a] * conj(g->fk_lv[b]);
				g->c_er[o] += g->fk_rho[b] * conj(g->fk_e[a]);
				g->c_jr[o] += g->fk_rho[b] * conj(g->fk_lv[a]);
				g->c_je[o] += g->fk_e[b] * conj(g->fk_lv[a]);
				g->c_X[o] += g->fk_X[a] * conj(g->fk_lv[b]);
			}
		}
	g->nsample++;
	static const char *names[11] = {"gh-rho-acf.dat", "gh-trans-momentum-acf.dat", "gh-long-momentum-acf.dat",
					"gh-energy-acf.dat", "gh-rho-energy-ccf.dat", "gh-rho-long-momentum-ccf.dat",
					"gh-energy-long-momentum-ccf.dat", "gh-energy-rho-ccf.dat",
					"gh-long-momentum-rho-ccf.dat", "gh-long-momentum-energy-ccf.dat", "gh-X-acf.dat"};
	double complex *cs[11] = {g->c_scatt, g->c_tv, g->c_lv, g->c_e, g->c_re, g->c_rj, g->c_ej, g->c_er, g->c_jr,
				  g->c_je, g->c_X};
	for (int f = 0; f < 11; f++) {
		FILE *fp = fopen(names[f], "w");
		if (!fp) sep_error("%s: Error opening files", __func__);
		for (int n = 0; n < lv; n++) {
			fprintf(fp, "%f ", n * g->dtsample);
			const double fac = 1.0 / (g->nsample * sys.volume * (lv - n));
			for (int k = 0; k < nk; k++) {
				const double complex v = cs[f][(size_t)n * nk + k] * fac;
				fprintf(fp, "%f %f ", creal(v), cimag(v));
			}
			fprintf(fp, "\n");
		}
		fclose(fp);
	}
	g->i = 0;
}

/* ---- mmsd: source/sepsampler.c:1958-2036 ---- */
static void mmsd_sample(struct sepmmsd *p, seppart *pptr, sepmol *mols, sepsys sys)
{
	rt_ctx *c = sampler_ctx(pptr, &sys);
	if (p->ctx != c) {
		if (p->dev) sepdev_mmsd_destroy(p->dev);
		p->dev = NULL;
	}
	mol_tables(&p->tab, &p->ctx, c, mols, &sys);
	if (!p->dev) rt_check(sepdev_mmsd_create(c->dev, p->tab, p->nk, p->k, &p->dev), "mmsd sampler");
	int ntype = 0;
	for (int n = 0; n < p->nmol; n++) {
		p->sel[n] = mols[n].type == p->type;
		ntype += p->sel[n];
	}
	int index = p->i;
	rt_check(sepdev_mmsd_sample(c->dev, p->tab, p->dev, p->sel, index == 0, p->out), "mmsd sample");
	p->msd[index] += p->out[0];
	for (int j = 0; j < p->nk; j++) p->Fs[(size_t)index * p->nk + j] += p->out[1 + j];
	index++;
	if (index == p->lvec) {
		p->nsample++;
		FILE *f = fopen("mmsd.dat", "w");
		if (!f) sep_error("%s: Couldn't open file", __func__);
		for (int n = 0; n < p->lvec; n++) fprintf(f, "%f %f \n", n * p->dtsample, p->msd[n] / (ntype * p->nsample));
		fclose(f);
		f = fopen("mmsd-incoherent.dat", "w");
		if (!f) sep_error("%s: Couldn't open file", __func__);
		for (int n = 0; n < p->lvec; n++) {
			fprintf(f, "%f ", n * p->dtsample);
			for (int j = 0; j < p->nk; j++) fprintf(f, "%f ", p->Fs[(size_t)n * p->nk + j] / (p->nsample * ntype));
			fprintf(f, "\n");
		}
		fclose(f);
		index = 0;
	}
	p->i = index;
}

/* source/sepsampler.c:2107-2114 */
void sep_set_inter_scatt(sepsampler *sampler)
{
	if (sampler->flag_scatt == 1) sampler->scatt[0]->intropt = 'i';
	else sep_error("%s: Couldn't set option since scatt in not initialized", __func__);
}

/* ---- scatt: source/sepsampler.c:2142-2213 ---- */
static void scatt_sample(struct sepscatt *p, seppart *pptr, sepsys sys)
{
	rt_ctx *c = sampler_ctx(pptr, &sys);
	/* the requested types by their first position in the string */
	int umap[SEPDEV_MAXTYPES], first[8];
	for (int t = 0; t < SEPDEV_MAXTYPES; t++) umap[t] = -1;
	for (int u = 0; u < p->ntypes; u++) {
		first[u] = u;
		for (int v = 0; v < u; v++)
			if (p->types[v] == p->types[u]) { first[u] = first[v]; break; }
		const int tid = rt_type_id(c, p->types[u]);
		if (tid >= 0 && first[u] == u) umap[tid] = u;
	}
	const int inter = p->intropt == 'i', ncl = inter ? 2 : 1;
	const int nv = 2 * p->ntypes * ncl, nk = p->nk;
	rt_check(sepdev_scatt(c->dev, nk, p->ntypes, ncl, umap, p->out), "scatt sample");
	int cb = 0;
	for (int a = 0; a < p->ntypes; a++)
		for (int b = a; b < p->ntypes; b++, cb++)
			for (int j = 0; j < nk; j++) {
				const double *o = p->out + (size_t)j * nv;
				const int qa = 2 * (first[a] * ncl + 0), qb = 2 * (first[b] * ncl + (inter ? 1 : 0));
				const size_t at = ((size_t)cb * p->lvec + p->index) * nk + j;
				p->p1[at] = o[qa] + I * o[qa + 1];
				p->m2[at] = o[qb] - I * o[qb + 1];
			}
	p->index++;
	if (p->index < p->lvec) return;
	p->index = 0;
	p->nsample++;
	const int lv = p->lvec;
	cb = 0;
	for (int a = 0; a < p->ntypes; a++)
		for (int b = a; b < p->ntypes; b++, cb++) {
			const size_t base = (size_t)cb * lv * nk;
			for (int k = 0; k < nk; k++)
				for (int n = 0; n < lv; n++)
					for (int m = 0; m < lv - n; m++)
						p->sc[base + (size_t)n * nk + k] +=
							p->p1[base + (size_t)m * nk + k] * p->m2[base + (size_t)(n + m) * nk + k];
			char name[64];
			snprintf(name, sizeof name, "scatt-%c%c.dat", p->types[a], p->types[b]);
			FILE *f = fopen(name, "w");
			if (!f) sep_error("Couldn't open file");
			const double dt = p->tspan / lv;
			for (int n = 0; n < lv; n++) {
				fprintf(f, "%f ", n * dt);
				const double fac = 1.0 / (p->nsample * sys.volume * (lv - n));
				for (int k = 0; k < nk; k++) fprintf(f, "%f ", creal(p->sc[base + (size_t)n * nk + k] * fac));
				fprintf(f, "\n");
			}
			fclose(f);
		}
}

/* w solving in w = s by Gaussian elimination with partial pivoting */
static void solve3(double w[3], const double s[3], const double in[9])
{
	double a[3][4];
	for (int r = 0; r < 3; r++) {
		for (int c = 0; c < 3; c++) a[r][c] = in[3 * r + c];
		a[r][3] = s[r];
	}
	for (int c = 0; c < 3; c++) {
		int piv = c;
		for (int r = c + 1; r < 3; r++)
			if (fabs(a[r][c]) > fabs(a[piv][c])) piv = r;
		if (piv != c)
			for (int k = 0; k < 4; k++) { const double t = a[c][k]; a[c][k] = a[piv][k]; a[piv][k] = t; }
		for (int r = c + 1; r < 3; r++) {
			const double f = a[r][c] / a[c][c];
			for (int k = c; k < 4; k++) a[r][k] -= f * a[c][k];
		}
	}
	for (int r = 2; r >= 0; r--) {
		double t = a[r][3];
		for (int k = r + 1; k < 3; k++) t -= a[r][k] * w[k];
		w[r] = t / a[r][r];
	}
}

/* ---- mprofs: source/sepsampler.c:1571-1666 ----
 * The bin of a molecule is floor(x_cm / dl), the last bin for a centre at
 * the box edge (where the reference ends the program). */
static void mprofs_sample(struct sepmprofs *p, seppart *pptr, sepmol *mols, sepsys sys)
{
	rt_ctx *c = sampler_ctx(pptr, &sys);
	mol_tables(&p->tab, &p->ctx, c, mols, &sys);
	for (int n = 0; n < p->nmol; n++) p->sel[n] = mols[n].type == p->type;
	rt_check(sepdev_mprofs(c->dev, p->tab, p->sel, p->dir, p->dirvel, p->lvec, p->out), "mprofs");
	for (int k = 0; k < 16 * p->lvec; k++) p->acc[k] += p->out[k];
	p->nsample++;
	if (p->nsample % 100 != 0) return;
	const int dir = p->dir;
	const double dl = sys.length[dir] / p->lvec;
	double dV;
	if (dir == 0) dV = dl * sys.length[1] * sys.length[2];
	else if (dir == 1) dV = sys.length[0] * dl * sys.length[2];
	else dV = sys.length[0] * sys.length[1] * dl;
	FILE *f = fopen("mprofs.dat", "w");
	if (!f) sep_error("%s: Couldn't open file", __func__);
	const double fac = 1 / (p->nsample * dV);
	for (int n = 0; n < p->lvec; n++) {
		const double *q = p->acc + 16 * (size_t)n;
		const double x = (n + 0.5) * dl;
		if (q[2] > 0) {
			const double a = q[1] * fac, b = q[0] * fac;
			const double av_numb = q[2] / p->nsample;
			const double tc = q[6] / (2 * p->nsample * av_numb);
			double spin[3], in[9], w[3] = {0.0, 0.0, 0.0};
			for (int k = 0; k < 3; k++) spin[k] = q[3 + k] * fac;
			for (int k = 0; k < 9; k++) in[k] = q[7 + k] * fac;
			solve3(w, spin, in);
			fprintf(f, "%e %e %e %e %e ", x, a, b / a, tc, w[p->diramom]);
			fprintf(f, "%e %e %e %e %e %e %e %e %e %e %e %e\n", spin[0], spin[1], spin[2], in[0], in[1],
				in[2], in[3], in[4], in[5], in[6], in[7], in[8]);
		} else {
			/* the reference's empty-bin line, spacing included */
			fprintf(f, "%e %e %e %e %e %e ", x, 0.0, 0.0, 0.0, 0.0, 0.0);
			fprintf(f, "%e %e % e%e %e %e %e %e %e %e %e %e\n", 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,
				0.0, 0.0, 0.0);
		}
	}
	fclose(f);
}

/* ---- radial: source/sepsampler.c:396-461 ---- */
static void radial_sample(struct sepradial *p, seppart *pptr, sepsys sys)
{
	rt_ctx *c = sampler_ctx(pptr, &sys);
	const int nt = c->ntypes > 0 ? c->ntypes : 1;
	for (int a = 0; a < nt; a++)
		for (int b = 0; b < nt; b++) {
			unsigned m = 0;
			int cc = 0;
			for (int t1 = 0; t1 < p->ntypes; t1++)
				for (int t2 = t1; t2 < p->ntypes; t2++, cc++)
					if ((c->tchar[a] == p->types[t1] && c->tchar[b] == p->types[t2]) ||
					    (c->tchar[a] == p->types[t2] && c->tchar[b] == p->types[t1]))
						m |= 1u << cc;
			p->mask[a * nt + b] = m;
		}
	rt_check(sepdev_radial(c->dev, p->lvec, p->ncomb, nt, p->mask, p->out), "radial distribution");
	for (int k = 0; k < p->lvec * p->ncomb; k++) p->hist[k] += p->out[k];
	p->nsample++;
	const double dg = 0.5 * sys.length[0] / p->lvec;
	FILE *f = fopen("radial.dat", "w");
	if (!f) sep_error("%s: Couldn't open file", __func__);
	for (int i = 0; i < p->lvec; i++) {
		const double vi = pow(i * dg, 3.0), vii = pow((i + 1) * dg, 3.0);
		fprintf(f, "%f ", (i + 0.5) * dg);
		for (int n = 0; n < p->ncomb; n++) {
			const double fac = 1.0 / ((vii - vi) * p->nsample);
			fprintf(f, "%f ", p->hist[(size_t)i * p->ncomb + n] * fac);
		}
		fprintf(f, "\n");
	}
	fclose(f);
}

/* source/sepsampler.c:177-240 (the samplers provided here, in its order) */
void sep_sample(seppart *pptr, sepsampler *sptr, sepret *ret, sepsys sys, unsigned n)
{
	if (sptr->flag_sacf == 1 && n % sptr->sacf->isample == 0) sacf_sample(sptr->sacf, ret, sys);
	if (sptr->flag_vacf == 1 && n % sptr->vacf->isample == 0) vacf_sample(sptr->vacf, pptr, sys);
	if (sptr->flag_msacf == 1 && n % sptr->msacf->isample == 0)
		msacf_sample(sptr->msacf, pptr, sptr->molptr, ret, sys);
	if (sptr->flag_gh == 1 && n % sptr->gh->isample == 0) gh_sample(sptr->gh, pptr, sys);
	if (sptr->flag_mgh == 1 && n % sptr->mgh->isample == 0) mgh_sample(sptr->mgh, pptr, sptr->molptr, sys);
	if (sptr->flag_profs == 1 && n % sptr->profs->isample == 0) profs_sample(sptr->profs, pptr, sys);
	if (sptr->flag_mprofs == 1 && n % sptr->mprofs->isample == 0)
		mprofs_sample(sptr->mprofs, pptr, sptr->molptr, sys);
	if (sptr->flag_mvacf == 1 && n % sptr->mvacf->isample == 0)
		mvacf_sample(sptr->mvacf, pptr, sptr->molptr, sys);
	if (sptr->flag_mavacf == 1 && n % sptr->mavacf->isample == 0)
		mavacf_sample(sptr->mavacf, pptr, sptr->molptr, sys);
	if (sptr->flag_radial == 1 && n % sptr->radial->isample == 0) radial_sample(sptr->radial, pptr, sys);
	if (sptr->flag_msd == 1) {
		struct sepmsd *m = sptr->msd;
		/* crossings: counted exactly on the device at every step */
		if (!m->logflag && n % m->isample == 0) {
			msd_sample(m, pptr, sys);
		} else if (m->logflag && sptr->msd_counter % m->logcounter == 0) {
			msd_sample(m, pptr, sys);
			m->logcounter = m->i == 0 ? 1 : 2 * m->logcounter;
		}
		sptr->msd_counter++;
	}
	if (sptr->flag_mmsd == 1 && n % sptr->mmsd->isample == 0) mmsd_sample(sptr->mmsd, pptr, sptr->molptr, sys);
	if (sptr->flag_scatt == 1 && n % sptr->scatt[0]->isample == 0) scatt_sample(sptr->scatt[0], pptr, sys);
}

void sep_close_sampler(sepsampler *ptr)
{
	if (ptr->flag_sacf == 1) {
		free(ptr->sacf->sacf);
		free(ptr->sacf->stress);
		free(ptr->sacf);
	}
	if (ptr->flag_vacf == 1) {
		if (ptr->vacf->dev) sepdev_vacf_destroy(ptr->vacf->dev);
		free(ptr->vacf->vacf);
		free(ptr->vacf->block);
		free(ptr->vacf);
	}
	if (ptr->flag_mavacf == 1) {
		struct sepmavacf *p = ptr->mavacf;
		if (p->dev) sepdev_vacf_destroy(p->dev);
		if (p->tab) sepdev_moltab_destroy(p->tab);
		free(p->vacf); free(p->block); free(p->sel);
		free(p);
	}
	if (ptr->flag_mprofs == 1) {
		struct sepmprofs *p = ptr->mprofs;
		if (p->tab) sepdev_moltab_destroy(p->tab);
		free(p->acc); free(p->out); free(p->sel);
		free(p);
	}
	if (ptr->flag_scatt == 1) {
		struct sepscatt *p = ptr->scatt[0];
		free(p->p1); free(p->m2); free(p->sc); free(p->out);
		free(p);
		free(ptr->scatt);
	}
	if (ptr->flag_mmsd == 1) {
		struct sepmmsd *p = ptr->mmsd;
		if (p->dev) sepdev_mmsd_destroy(p->dev);
		if (p->tab) sepdev_moltab_destroy(p->tab);
		free(p->k); free(p->msd); free(p->Fs); free(p->out); free(p->sel);
		free(p);
	}
	if (ptr->flag_gh == 1) {
		struct sepgh *g = ptr->gh;
		if (g->dev) sepdev_gh_destroy(g->dev);
		double complex *arr[] = {g->fk_tv, g->fk_lv, g->fk_rho, g->fk_e, g->fk_X, g->c_tv, g->c_lv, g->c_scatt,
					 g->c_e, g->c_re, g->c_rj, g->c_ej, g->c_er, g->c_jr, g->c_je, g->c_X};
		for (size_t q = 0; q < sizeof arr / sizeof arr[0]; q++) free(arr[q]);
		free(g->k); free(g->out);
		free(g);
	}
	if (ptr->flag_radial == 1) {
		free(ptr->radial->hist); free(ptr->radial->out); free(ptr->radial->mask);
		free(ptr->radial);
	}
	if (ptr->flag_profs == 1) {
		struct sepprofs *p = ptr->profs;
		free(p->momc); free(p->svel); free(p->dens); free(p->temp); free(p->hist);
		free(p);
	}
	if (ptr->flag_msacf == 1) {
		free(ptr->msacf->sacf); free(ptr->msacf->sstress); free(ptr->msacf->astress);
		free(ptr->msacf);
	}
	if (ptr->flag_mvacf == 1) {
		if (ptr->mvacf->dev) sepdev_vacf_destroy(ptr->mvacf->dev);
		if (ptr->mvacf->tab) sepdev_moltab_destroy(ptr->mvacf->tab);
		free(ptr->mvacf->vacf); free(ptr->mvacf->block);
		free(ptr->mvacf);
	}
	if (ptr->flag_mgh == 1) {
		struct sepmgh *g = ptr->mgh;
		if (g->tab) sepdev_moltab_destroy(g->tab);
		double complex *arr[] = {g->fk_tv, g->fk_lv, g->fk_rho, g->fk_tav, g->fk_lav, g->fk_e, g->fk_dip,
					 g->fk_X, g->c_tv, g->c_lv, g->c_scatt, g->c_tav, g->c_lav, g->c_e,
					 g->c_vav, g->c_dip, g->c_X};
		for (size_t q = 0; q < sizeof arr / sizeof arr[0]; q++) free(arr[q]);
		free(g->k); free(g->out);
		free(g);
	}
	if (ptr->flag_msd == 1) {
		struct sepmsd *m = ptr->msd;
		if (m->dev) sepdev_msd_destroy(m->dev);
		free(m->msd); free(m->msdsq); free(m->time); free(m->k); free(m->Fs); free(m->out);
		free(m);
	}
	memset(ptr, 0, sizeof *ptr);
}
