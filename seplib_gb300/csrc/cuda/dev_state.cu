// dev_state.cu - context lifetime, host<->device transfers, slots, events.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "dev_common.cuh"
#include "dev_decide.cuh"

static char g_err[512];

extern "C" void sepdev_set_error(const char *what, cudaError_t e)
{
	snprintf(g_err, sizeof g_err, "%s: %s (%d)", what, cudaGetErrorString(e), (int)e);
}

extern "C" const char *sepdev_last_error(void) { return g_err; }

extern "C" int sepdev_device_count(void)
{
	int n = 0;
	if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
	return n;
}

template <class T>
static int dalloc(T **p, size_t count)
{
	*p = NULL;
	if (count == 0) count = 1;
	cudaError_t e = cudaMalloc((void **)p, sizeof(T) * count);
	if (e != cudaSuccess) { sepdev_set_error("cudaMalloc", e); return SEPDEV_ENOMEM; }
	return SEPDEV_OK;
}

#define DA(p, c) do { int r_ = dalloc(&(p), (c)); if (r_) { sepdev_destroy(d); return r_; } } while (0)

extern "C" int sepdev_create(sepdev **out, long n)
{
	*out = NULL;
	if (n <= 0) return SEPDEV_EINVAL;
	if (sepdev_device_count() < 1) {
		snprintf(g_err, sizeof g_err, "no CUDA device visible");
		return SEPDEV_ENODEV;
	}
	sepdev *d = (sepdev *)calloc(1, sizeof(sepdev));
	if (!d) return SEPDEV_ENOMEM;
	d->n = n;
	CK(cudaGetDevice(&d->device));
	CK(cudaStreamCreateWithFlags(&d->st, cudaStreamNonBlocking));
	for (int k = 0; k < SEPDEV_NEV; k++) CK(cudaEventCreate(&d->ev[k]));
	DA(d->pos[0], n); DA(d->pos[1], n);
	DA(d->xlo, n); DA(d->xlo_b, n);
	DA(d->vhi, n); DA(d->vhi_b, n);
	DA(d->vlo, n); DA(d->vlo_b, n);
	DA(d->frc, n); DA(d->frc_b, n);
	DA(d->xn, n);
	DA(d->cross, n); DA(d->cross_b, n);
	DA(d->cbase, n); DA(d->cbase_b, n);
	DA(d->gid, n); DA(d->gid_b, n); DA(d->inv, n);
	DA(d->charge, n); DA(d->charge_b, n);
	DA(d->mol, n); DA(d->mol_b, n);
	DA(d->cellof, n); DA(d->celloff, n); DA(d->perm, n);
	DA(d->ncnt, n);
	DA(d->d_ps, 1);
	d->nslots = 16;
	DA(d->slots, (size_t)d->nslots * SLOT_FIELDS);
	DA(d->flags, 4);
	DA(d->take_arrive, 1);
	d->take_ready = -1;
	CK(cudaHostAlloc((void **)&d->h_slots, sizeof(long long) * d->nslots * SLOT_FIELDS, cudaHostAllocMapped));
	CK(cudaHostAlloc((void **)&d->h_flags, sizeof(unsigned) * 4, cudaHostAllocMapped));
	CK(cudaHostGetDevicePointer((void **)&d->hd_slots, d->h_slots, 0));
	CK(cudaHostGetDevicePointer((void **)&d->hd_flags, d->h_flags, 0));
	CK(cudaMemsetAsync(d->slots, 0, sizeof(long long) * d->nslots * SLOT_FIELDS, d->st));
	CK(cudaMemsetAsync(d->flags, 0, sizeof(unsigned) * 4, d->st));
	CK(cudaMemsetAsync(d->take_arrive, 0, sizeof(unsigned), d->st));
	CK(cudaMemsetAsync(d->frc, 0, sizeof(float4) * n, d->st));
	d->team = 1;
	d->groups = 2;
	d->cellf = 1.0;
	CK(cudaDeviceGetAttribute(&d->nsm, cudaDevAttrMultiProcessorCount, d->device));
	{
		// in-place transfers need device access to pageable host memory
		// (GB300: coherent NVLink-C2C through the host page tables);
		// SEPLIB_HOSTIO=staged selects the staged copies regardless
		int pma = 0;
		CK(cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, d->device));
		const char *hio = getenv("SEPLIB_HOSTIO");
		d->hostio_direct = pma == 1 && !(hio && strcmp(hio, "staged") == 0);
	}
	*out = d;
	return SEPDEV_OK;
}

extern void sepdev_runner_free(sepdev *d);

extern "C" void sepdev_destroy(sepdev *d)
{
	if (!d) return;
	if (d->st) cudaStreamSynchronize(d->st);
	sepdev_runner_free(d);
	void *bufs[] = {d->pos[0], d->pos[1], d->xlo, d->xlo_b, d->vhi, d->vhi_b, d->vlo, d->vlo_b,
			d->frc, d->frc_b, d->xn, d->cross, d->cross_b, d->cbase, d->cbase_b, d->gid,
			d->gid_b, d->inv, d->charge, d->charge_b, d->mol, d->mol_b, d->cellof,
			d->celloff, d->cellcount, d->cellstart, d->perm, d->nl, d->ncnt, d->exb_start,
			d->exb_idx, d->exa_start, d->exa_idx, d->bonds, d->angles, d->diheds_abcd,
			d->dihed_type, d->inc_start, d->inc_term, d->term_out, d->slots, d->flags, d->take_arrive,
			d->d_ps, d->flush_buf, d->hio_scr, d->x0, d->tscr};
	for (size_t k = 0; k < sizeof bufs / sizeof bufs[0]; k++)
		if (bufs[k]) cudaFree(bufs[k]);
	for (int k = 0; k < SEPDEV_MAXTAB; k++)
		if (d->tab[k]) cudaFree(d->tab[k]);
	for (int k = 0; k < SEPDEV_NEXT; k++) {
		if (d->ext[k]) cudaFree(d->ext[k]);
		if (d->ext_b[k]) cudaFree(d->ext_b[k]);
	}
	{
		void *mv[] = {d->mv_first, d->mv_nuau, d->mv_start, d->mv_atoms, d->mv_mass, d->mv_cm,
			      d->mv_finter, d->mv_out};
		for (size_t k = 0; k < sizeof mv / sizeof mv[0]; k++)
			if (mv[k]) cudaFree(mv[k]);
	}
	if (d->h_slots) cudaFreeHost(d->h_slots);
	if (d->stage) cudaFreeHost(d->stage);
	if (d->h_flags) cudaFreeHost(d->h_flags);
	for (int k = 0; k < SEPDEV_NEV; k++)
		if (d->ev[k]) cudaEventDestroy(d->ev[k]);
	if (d->st) cudaStreamDestroy(d->st);
	free(d);
}

// ---- number-format conversions on the host ---------------------------------

// x -> 64-bit fixed-point fraction of L (wrapped into [0, L))
static void to_fixed(double x, double L, unsigned *hi, unsigned *lo)
{
	double fr = x / L;
	fr -= floor(fr);
	if (fr >= 1.0) fr = 0.0;
	double t = ldexp(fr, 32);
	double h = floor(t);
	double r = ldexp(t - h, 32);
	*hi = (unsigned)h;
	*lo = (unsigned)floor(r);
}

static double from_fixed(unsigned hi, unsigned lo, double L)
{
	return (ldexp((double)hi, -32) + ldexp((double)lo, -64)) * L;
}

// Pinned staging for uploads and downloads, kept by the context: pinning
// tens of megabytes costs milliseconds, so it is done once, not per call.
// Arrays are carved out of one block in 256-byte aligned pieces.
struct Stage {
	char *base;
	size_t off;
	template <class T> T *take(long n)
	{
		T *p = (T *)(base + off);
		off += ((sizeof(T) * (size_t)n + 255) & ~(size_t)255);
		return p;
	}
};

static int stage_get(sepdev *d, size_t bytes, Stage *st)
{
	if (d->stage_bytes < bytes) {
		if (d->stage) { cudaFreeHost(d->stage); d->stage = NULL; d->stage_bytes = 0; }
		cudaError_t e = cudaMallocHost(&d->stage, bytes);
		if (e != cudaSuccess) { sepdev_set_error("cudaMallocHost(staging)", e); return SEPDEV_ENOMEM; }
		d->stage_bytes = bytes;
	}
	st->base = (char *)d->stage;
	st->off = 0;
	return SEPDEV_OK;
}

// upper bound of the staging bytes of one upload or download of n particles
static size_t stage_need(long n)
{
	return 12 * (((size_t)n * 16 + 255) & ~(size_t)255);
}

extern "C" int sepdev_upload(sepdev *d, const double *x, const double *v, const double *f,
			     const double *m, const double *z, const int *type_id,
			     const int *molindex, const int *crossings, const int *cross_neighb,
			     const double *L)
{
	const long n = d->n;
	for (int k = 0; k < 3; k++) {
		if (!(L[k] > 0.0)) return SEPDEV_EINVAL;
		d->L[k] = L[k];
		d->fscale[k] = (float)(L[k] / 4294967296.0);
	}
	Stage sg;
	int rc = stage_get(d, stage_need(n), &sg);
	if (rc) return rc;
	int4 *hp = sg.take<int4>(n); uint4 *hl = sg.take<uint4>(n);
	float4 *hvh = sg.take<float4>(n), *hvl = sg.take<float4>(n), *hf = sg.take<float4>(n);
	int4 *hc = sg.take<int4>(n), *hb = sg.take<int4>(n);
	int *hg = sg.take<int>(n), *hm = sg.take<int>(n); float *hq = sg.take<float>(n);
	d->has_charge = 0;
	for (long i = 0; i < n; i++) {
		unsigned h[3], l[3];
		for (int k = 0; k < 3; k++) to_fixed(x[3 * i + k], L[k], &h[k], &l[k]);
		hp[i] = make_int4((int)h[0], (int)h[1], (int)h[2], type_id ? type_id[i] : 0);
		hl[i] = make_uint4(l[0], l[1], l[2], 0u);
		float vh[3], vl[3];
		for (int k = 0; k < 3; k++) {
			vh[k] = (float)v[3 * i + k];
			vl[k] = (float)(v[3 * i + k] - (double)vh[k]);
		}
		double mi = m ? m[i] : 1.0;
		hvh[i] = make_float4(vh[0], vh[1], vh[2], (float)mi);
		hvl[i] = make_float4(vl[0], vl[1], vl[2], (float)(1.0 / mi));
		hf[i] = f ? make_float4((float)f[3 * i], (float)f[3 * i + 1], (float)f[3 * i + 2], 0.f)
			  : make_float4(0.f, 0.f, 0.f, 0.f);
		int c[3] = {0, 0, 0}, cn[3] = {0, 0, 0};
		for (int k = 0; k < 3; k++) {
			if (crossings) c[k] = crossings[3 * i + k];
			if (cross_neighb) cn[k] = cross_neighb[3 * i + k];
		}
		hc[i] = make_int4(c[0], c[1], c[2], 0);
		hb[i] = make_int4(c[0] - cn[0], c[1] - cn[1], c[2] - cn[2], 0);
		hg[i] = (int)i;
		hm[i] = molindex ? molindex[i] : -1;
		hq[i] = z ? (float)z[i] : 0.f;
		if (z && fabs(z[i]) >= 2.220446049250313e-16) d->has_charge = 1;
	}
	d->cur = 0;
#define UP(dst, src) if ((rc = (cudaMemcpyAsync(dst, src, sizeof(*(src)) * n, cudaMemcpyHostToDevice, d->st) == cudaSuccess) ? 0 : SEPDEV_ECUDA)) goto done
	UP(d->pos[0], hp); UP(d->xlo, hl); UP(d->vhi, hvh); UP(d->vlo, hvl); UP(d->frc, hf);
	UP(d->cross, hc); UP(d->cbase, hb); UP(d->gid, hg); UP(d->inv, hg); UP(d->mol, hm);
	UP(d->charge, hq); UP(d->xn, hp);
#undef UP
	if (cudaStreamSynchronize(d->st) != cudaSuccess) rc = SEPDEV_ECUDA;
	d->list_valid = 0;
done:
	if (rc == SEPDEV_ECUDA) sepdev_set_error("upload", cudaGetLastError());
	return rc;
}

extern "C" int sepdev_download(sepdev *d, double *x, double *v, double *f, int *crossings,
			       int *cross_neighb, double *xn)
{
	const long n = d->n;
	Stage sg;
	int rc = stage_get(d, stage_need(n), &sg);
	if (rc) return rc;
	int4 *hp = sg.take<int4>(n), *hc = sg.take<int4>(n), *hb = sg.take<int4>(n);
	int4 *hx = sg.take<int4>(n); uint4 *hl = sg.take<uint4>(n);
	float4 *hvh = sg.take<float4>(n), *hvl = sg.take<float4>(n), *hf = sg.take<float4>(n);
	int *hg = sg.take<int>(n);
#define DN(dst, src) if ((rc = (cudaMemcpyAsync(dst, src, sizeof(*(dst)) * n, cudaMemcpyDeviceToHost, d->st) == cudaSuccess) ? 0 : SEPDEV_ECUDA)) goto done
	DN(hp, d->pos[d->cur]); DN(hl, d->xlo); DN(hvh, d->vhi); DN(hvl, d->vlo); DN(hf, d->frc);
	DN(hc, d->cross); DN(hb, d->cbase); DN(hg, d->gid); DN(hx, d->xn);
#undef DN
	if (cudaStreamSynchronize(d->st) != cudaSuccess) { rc = SEPDEV_ECUDA; goto done; }
	for (long s = 0; s < n; s++) {
		long u = hg[s];
		if (u < 0 || u >= n) { rc = SEPDEV_EINVAL; goto done; }
		const unsigned ph[3] = {(unsigned)hp[s].x, (unsigned)hp[s].y, (unsigned)hp[s].z};
		const unsigned pl[3] = {hl[s].x, hl[s].y, hl[s].z};
		const float vh[3] = {hvh[s].x, hvh[s].y, hvh[s].z}, vl[3] = {hvl[s].x, hvl[s].y, hvl[s].z};
		const float ff[3] = {hf[s].x, hf[s].y, hf[s].z};
		const int cc[3] = {hc[s].x, hc[s].y, hc[s].z}, cb[3] = {hb[s].x, hb[s].y, hb[s].z};
		const unsigned xh[3] = {(unsigned)hx[s].x, (unsigned)hx[s].y, (unsigned)hx[s].z};
		for (int k = 0; k < 3; k++) {
			if (x) x[3 * u + k] = from_fixed(ph[k], pl[k], d->L[k]);
			if (v) v[3 * u + k] = (double)vh[k] + (double)vl[k];
			if (f) f[3 * u + k] = (double)ff[k];
			if (crossings) crossings[3 * u + k] = cc[k];
			if (cross_neighb) cross_neighb[3 * u + k] = cc[k] - cb[k];
			if (xn) xn[3 * u + k] = from_fixed(xh[k], 0u, d->L[k]);
		}
	}
done:
	if (rc == SEPDEV_ECUDA) sepdev_set_error("download", cudaGetLastError());
	return rc;
}

// ---- sum m v^2 -----------------------------------------------------------
__global__ void k_sumv2(long n, const float4 *__restrict__ vhi, const float4 *__restrict__ vlo,
			long long *slot)
{
	float acc[1] = {0.f};
	for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
		float4 a = vhi[i], b = vlo[i];
		float vx = a.x + b.x, vy = a.y + b.y, vz = a.z + b.z;
		acc[0] += a.w * (vx * vx + vy * vy + vz * vz);
	}
	const int fld[1] = {SLOT_SUMV2};
	block_to_slot<1>(acc, fld, slot, 0.f, -1);
}

extern "C" int sepdev_sumv2(sepdev *d, double *out)
{
	long long *slot = d->slots + (size_t)(d->nslots - 1) * SLOT_FIELDS;
	CK(cudaMemsetAsync(slot, 0, sizeof(long long) * SLOT_FIELDS, d->st));
	k_sumv2<<<152 * 4, 256, 0, d->st>>>(d->n, d->vhi, d->vlo, slot);
	CKL(d);
	long long h;
	CK(cudaMemcpyAsync(&h, slot + SLOT_SUMV2, sizeof h, cudaMemcpyDeviceToHost, d->st));
	CK(cudaStreamSynchronize(d->st));
	*out = (double)h * FX_ISCALE;
	return SEPDEV_OK;
}

// ---- slots -----------------------------------------------------------------
extern "C" int sepdev_slots_reset(sepdev *d)
{
	CK(cudaMemsetAsync(d->slots, 0, sizeof(long long) * d->nslots * SLOT_FIELDS, d->st));
	return SEPDEV_OK;
}

// The read-back as a kernel of its own (one block; see take_copy).
__global__ void k_slots_take(TakeArgs t)
{
	take_copy(t, threadIdx.x, blockDim.x);
}

extern "C" int sepdev_slots_take(sepdev *d, int nslots, double *out, unsigned *flags, int keep_on_overflow)
{
	if (nslots < 0 || nslots > d->nslots) return SEPDEV_EINVAL;
	const int ready = d->take_ready;
	d->take_ready = -1;
	if (ready >= 0) {
		// the step kernel handed its slots over (and cleared them unless its
		// list overflowed); a read of other slots would find them cleared
		if (ready != nslots) return SEPDEV_EINVAL;
		CK(cudaStreamSynchronize(d->st));
		if (!keep_on_overflow && (d->h_flags[0] & 1u))
			CK(cudaMemsetAsync(d->slots, 0, sizeof(long long) * d->nslots * SLOT_FIELDS, d->st));
	} else {
		TakeArgs t;
		t.h = d->hd_slots;
		t.hf = d->hd_flags;
		t.arrive = NULL;
		t.slots = d->slots;
		t.flags = d->flags;
		t.nread = nslots;
		t.nall = d->nslots;
		t.keep = keep_on_overflow;
		k_slots_take<<<1, 512, 0, d->st>>>(t);
		CKL(d);
		CK(cudaStreamSynchronize(d->st));
	}
	// an unchecked list that did not overflow is settled by this read
	if (d->list_unchecked && !(d->h_flags[0] & 1u)) d->list_unchecked = 0;
	for (int s = 0; s < nslots; s++)
		for (int k = 0; k < SLOT_FIELDS; k++) {
			long long v = d->h_slots[s * SLOT_FIELDS + k];
			if (k == SLOT_MAXD2) {
				unsigned u = (unsigned)v;
				float fv;
				memcpy(&fv, &u, sizeof fv);
				out[s * SLOT_FIELDS + k] = fv;
			} else {
				out[s * SLOT_FIELDS + k] = (double)v * FX_ISCALE;
			}
		}
	if (flags) for (int k = 0; k < 4; k++) flags[k] = d->h_flags[k];
	return SEPDEV_OK;
}

// ---- events ------------------------------------------------------------------
extern "C" int sepdev_sync(sepdev *d)
{
	CK(cudaStreamSynchronize(d->st));
	return SEPDEV_OK;
}

extern "C" int sepdev_event_record(sepdev *d, int e)
{
	if (e < 0 || e >= SEPDEV_NEV) return SEPDEV_EINVAL;
	CK(cudaEventRecord(d->ev[e], d->st));
	return SEPDEV_OK;
}

extern "C" int sepdev_event_elapsed(sepdev *d, int e0, int e1, float *ms)
{
	if (e0 < 0 || e0 >= SEPDEV_NEV || e1 < 0 || e1 >= SEPDEV_NEV) return SEPDEV_EINVAL;
	CK(cudaEventSynchronize(d->ev[e1]));
	CK(cudaEventElapsedTime(ms, d->ev[e0], d->ev[e1]));
	return SEPDEV_OK;
}

extern "C" long sepdev_launch_count(sepdev *d) { return d->launches; }

// ---- tables and exclusions ---------------------------------------------------
extern "C" int sepdev_set_table(sepdev *d, int t, int nt, double r2min, double dr2,
				const float *ft, const float *u)
{
	if (t < 0 || t >= SEPDEV_MAXTAB || nt < 2 || !(dr2 > 0)) return SEPDEV_EINVAL;
	if (d->tab[t]) { cudaFree(d->tab[t]); d->tab[t] = NULL; }
	float2 *h = (float2 *)malloc(sizeof(float2) * nt);
	if (!h) return SEPDEV_ENOMEM;
	for (int k = 0; k < nt; k++) h[k] = make_float2(ft[k], u[k]);
	cudaError_t e = cudaMalloc((void **)&d->tab[t], sizeof(float2) * nt);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(d->tab[t], h, sizeof(float2) * nt, cudaMemcpyHostToDevice, d->st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
	free(h);
	if (e != cudaSuccess) { sepdev_set_error("set_table", e); return SEPDEV_ECUDA; }
	d->tab_n[t] = nt;
	d->tab_r2min[t] = (float)r2min;
	d->tab_idr2[t] = (float)(1.0 / dr2);
	return SEPDEV_OK;
}

static int upload_ints(sepdev *d, int **dst, const int *src, long count)
{
	if (*dst) { cudaFree(*dst); *dst = NULL; }
	if (dalloc(dst, count)) return SEPDEV_ENOMEM;
	CK(cudaMemcpyAsync(*dst, src, sizeof(int) * (count ? count : 1), cudaMemcpyHostToDevice, d->st));
	return SEPDEV_OK;
}

extern "C" int sepdev_set_exclusions(sepdev *d, const int *bs, const int *bi, const int *as,
				     const int *ai)
{
	int rc;
	if ((rc = upload_ints(d, &d->exb_start, bs, d->n + 1))) return rc;
	if ((rc = upload_ints(d, &d->exb_idx, bi, bs[d->n]))) return rc;
	if ((rc = upload_ints(d, &d->exa_start, as, d->n + 1))) return rc;
	if ((rc = upload_ints(d, &d->exa_idx, ai, as[d->n]))) return rc;
	CK(cudaStreamSynchronize(d->st));
	d->has_excl = 1;
	d->list_valid = 0;
	return SEPDEV_OK;
}
