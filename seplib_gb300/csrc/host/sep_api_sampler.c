/*
 * sep_api_sampler.c - the sacf, vacf and msd samplers of the sep C API.
 *
 * Control flow, sampling intervals, normalisations and output files follow
 * the reference (source/sepsampler.c:4-242 dispatch, :280-351 sacf,
 * :471-641 msd, :658-714 vacf).  The stress autocorrelation works on the
 * sepret values the host already has after every sep_leapfrog; vacf and msd
 * keep their particle data on the GPU (dev_sampler.cu) and only their
 * per-sample or per-block sums come back to the host.
 */
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
	} else {
		va_end(args);
		sep_error("%s: sampler %s is not provided by this GPU implementation "
			  "(available: sacf, vacf, msd)", __func__, sampler);
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

/* source/sepsampler.c:177-240 (the samplers provided here) */
void sep_sample(seppart *pptr, sepsampler *sptr, sepret *ret, sepsys sys, unsigned n)
{
	if (sptr->flag_sacf == 1 && n % sptr->sacf->isample == 0) sacf_sample(sptr->sacf, ret, sys);
	if (sptr->flag_vacf == 1 && n % sptr->vacf->isample == 0) vacf_sample(sptr->vacf, pptr, sys);
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
	if (ptr->flag_msd == 1) {
		struct sepmsd *m = ptr->msd;
		if (m->dev) sepdev_msd_destroy(m->dev);
		free(m->msd); free(m->msdsq); free(m->time); free(m->k); free(m->Fs); free(m->out);
		free(m);
	}
	memset(ptr, 0, sizeof *ptr);
}
