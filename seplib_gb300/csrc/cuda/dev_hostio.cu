// dev_hostio.cu - uploads and downloads that read and write the seppart array
// in place, from device code.
//
// On GB300 the GPU reaches the Grace host's memory coherently over NVLink-C2C
// through the host page tables (cudaDevAttrPageableMemoryAccess = 1), so the
// program's own malloc'ed seppart array is addressable from a kernel.  An
// upload is then one kernel that reads each particle's fields (x, v, f, m,
// type, z, crossings, cross_neighb, molindex, xn: the first 156 bytes and the
// xn triple of the 568-byte record) and writes the device arrays with the
// same conversions as the host path (64-bit fixed point, float-float
// velocity); a download is one kernel that writes x, v, f, a, crossings,
// cross_neighb and xn back into the records.  No host pass over the
// array and no staging copy is needed.  Where the attribute is 0 the
// library uses the staged host path (dev_state.cu).
//
// Host-side bookkeeping that the staged path does in its loop is done here
// on the device and read back once:
//   - the type-character map (ids in order of first appearance) from the
//     first index of every character;
//   - sum m v^2 in FP64, summed per block in a fixed order and then over the
//     blocks in order (run-to-run identical);
//   - the largest squared displacement from the host xn (the reference's
//     pending-update test), and whether any charge is non-zero.
#include <math.h>
#include <stdlib.h>
#include <stddef.h>
#include <string.h>
#include "dev_common.cuh"
#include "sepstrct.h"

#define HIO_B 128

// The fields a transfer touches, as 8-byte words of the 568-byte record:
// the head (x, v, f, a, m, type, z, neighb, cross_neighb, crossings,
// molindex: bytes 0-159) and xn.  A block moves the words of its HIO_B
// consecutive records through shared memory, so every warp-wide access to
// host memory covers one or two contiguous runs of a record instead of 32
// records 568 bytes apart.
#define HW_HEAD 20
#define HW_XN 3
#define HW (HW_HEAD + HW_XN)
static_assert(sizeof(seppart) % 8 == 0, "seppart is a whole number of 8-byte words");
static_assert(offsetof(seppart, molindex) + sizeof(int) <= 8 * HW_HEAD, "head words");
static_assert(offsetof(seppart, xn) % 8 == 0, "xn word-aligned");
#define RW (sizeof(seppart) / 8)
#define XN_W (offsetof(seppart, xn) / 8)

// word q of the record block: record q / HW, head word or xn word
__device__ __forceinline__ long rec_word(long r0, int q, int *r, int *w)
{
	*r = q / HW;
	*w = q - *r * HW;
	return (r0 + *r) * (long)RW + (*w < HW_HEAD ? *w : XN_W + *w - HW_HEAD);
}

// the block's records [r0, r0 + cnt) into sm[HIO_B][HW]
__device__ __forceinline__ void rec_load(const seppart *p, long r0, int cnt, unsigned long long (*sm)[HW])
{
	const unsigned long long *g = (const unsigned long long *)p;
	for (int q = threadIdx.x; q < cnt * HW; q += HIO_B) {
		int r, w;
		const long gi = rec_word(r0, q, &r, &w);
		sm[r][w] = g[gi];
	}
}

// typed views of a staged record
#define SM_D(rec, field, k) (((const double *)(rec))[offsetof(seppart, field) / 8 + (k)])
#define SM_I(rec, field, k) (((const int *)(rec))[offsetof(seppart, field) / 4 + (k)])
#define SM_XN(rec, k) (((const double *)(rec))[HW_HEAD + (k)])

struct HioUp {
	const seppart *p;
	long n;
	double L[3];
	int4 *pos, *cross, *cbase, *xn;
	uint4 *xlo;
	float4 *vhi, *vlo, *frc;
	int *gid, *inv, *mol;
	float *charge;
	int *first;                 // [256] first index of each type character
	double *part;               // per-block sums of m v^2
	unsigned long long *maxd2;  // bits of the largest squared displacement (>= 0)
	unsigned *has_charge;
};


__global__ void __launch_bounds__(HIO_B) k_upload_parts(HioUp a)
{
	__shared__ unsigned long long sm[HIO_B][HW];
	__shared__ double red[HIO_B];
	const long r0 = blockIdx.x * (long)HIO_B;
	const int cnt = (int)min((long)HIO_B, a.n - r0);
	rec_load(a.p, r0, cnt, sm);
	__syncthreads();
	const long i = r0 + threadIdx.x;
	double q = 0.0;
	if (i < a.n) {
		const unsigned long long *rec = sm[threadIdx.x];
		unsigned h[3], l[3];
		double d2 = 0.0;
		float vh[3], vl[3];
		const double m = SM_D(rec, m, 0);
		for (int k = 0; k < 3; k++) {
			const double x = SM_D(rec, x, k), v = SM_D(rec, v, k);
			to_fixed_dev(x, a.L[k], h[k], l[k]);
			vh[k] = (float)v;
			vl[k] = (float)__dsub_rn(v, (double)vh[k]);
			q = __dadd_rn(q, __dmul_rn(__dmul_rn(v, v), m));
			double r = __dsub_rn(x, SM_XN(rec, k));
			if (r > 0.5 * a.L[k]) r = __dsub_rn(r, a.L[k]);
			else if (r < -0.5 * a.L[k]) r = __dadd_rn(r, a.L[k]);
			d2 = __dadd_rn(d2, __dmul_rn(r, r));
		}
		const unsigned char tc = ((const unsigned char *)rec)[offsetof(seppart, type)];
		atomicMin(&a.first[tc], (int)i);
		const int4 ph = make_int4((int)h[0], (int)h[1], (int)h[2], (int)tc);   // .w remapped later
		a.pos[i] = ph;
		a.xn[i] = ph;
		a.xlo[i] = make_uint4(l[0], l[1], l[2], 0u);
		a.vhi[i] = make_float4(vh[0], vh[1], vh[2], (float)m);
		a.vlo[i] = make_float4(vl[0], vl[1], vl[2], (float)__ddiv_rn(1.0, m));
		a.frc[i] = make_float4((float)SM_D(rec, f, 0), (float)SM_D(rec, f, 1), (float)SM_D(rec, f, 2), 0.f);
		const int c0 = SM_I(rec, crossings, 0), c1 = SM_I(rec, crossings, 1), c2 = SM_I(rec, crossings, 2);
		a.cross[i] = make_int4(c0, c1, c2, 0);
		a.cbase[i] = make_int4(c0 - SM_I(rec, cross_neighb, 0), c1 - SM_I(rec, cross_neighb, 1),
				       c2 - SM_I(rec, cross_neighb, 2), 0);
		a.gid[i] = (int)i;
		a.inv[i] = (int)i;
		a.mol[i] = SM_I(rec, molindex, 0);
		const double z = SM_D(rec, z, 0);
		a.charge[i] = (float)z;
		if (fabs(z) >= 2.220446049250313e-16) atomicOr(a.has_charge, 1u);
		atomicMax(a.maxd2, (unsigned long long)__double_as_longlong(d2));
	}
	// sum of q over the block, fixed tree order
	red[threadIdx.x] = q;
	__syncthreads();
	for (int s = HIO_B / 2; s > 0; s >>= 1) {
		if ((int)threadIdx.x < s) red[threadIdx.x] = __dadd_rn(red[threadIdx.x], red[threadIdx.x + s]);
		__syncthreads();
	}
	if (threadIdx.x == 0) a.part[blockIdx.x] = red[0];
}

__global__ void k_upload_sum(const double *part, int nb, double *out)
{
	if (threadIdx.x != 0 || blockIdx.x != 0) return;
	double s = 0.0;
	for (int b = 0; b < nb; b++) s = __dadd_rn(s, part[b]);
	*out = s;
}

struct TypeMap { int id[256]; };

__global__ void k_upload_types(long n, int4 *pos, int4 *xn, TypeMap m)
{
	const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
	if (i < n) {
		const int id = m.id[pos[i].w & 255];
		pos[i].w = id;
		xn[i].w = id;
	}
}

// small device scratch of the in-place transfers, kept by the context
static int hio_scratch(sepdev *d, size_t bytes, char **out)
{
	if (d->hio_bytes < bytes) {
		if (d->hio_scr) { CK(cudaFree(d->hio_scr)); d->hio_scr = NULL; d->hio_bytes = 0; }
		CK(cudaMalloc(&d->hio_scr, bytes));
		d->hio_bytes = bytes;
	}
	*out = (char *)d->hio_scr;
	return SEPDEV_OK;
}

extern "C" int sepdev_direct_io(const sepdev *d) { return d->hostio_direct; }

extern "C" int sepdev_upload_parts(sepdev *d, const void *parts, const double *L, int max_types,
				   char *tchar, int *ntypes, double *sumv2, double *maxd2)
{
	const long n = d->n;
	if (!d->hostio_direct) return SEPDEV_EINVAL;
	HioUp a;
	a.p = (const seppart *)parts;
	a.n = n;
	for (int k = 0; k < 3; k++) {
		if (!(L[k] > 0.0)) return SEPDEV_EINVAL;
		a.L[k] = L[k];
		d->L[k] = L[k];
		d->fscale[k] = (float)(L[k] / 4294967296.0);
	}
	const int nb = (int)((n + HIO_B - 1) / HIO_B);
	// scratch: first[256] ints | sum | maxd2 | has_charge | per-block sums
	const size_t need = 256 * sizeof(int) + 4 * sizeof(double) + sizeof(double) * (size_t)nb;
	char *scr = NULL;
	int rc = hio_scratch(d, need, &scr);
	if (rc) return rc;
	a.first = (int *)scr;
	double *sum = (double *)(scr + 256 * sizeof(int));
	a.maxd2 = (unsigned long long *)(sum + 1);
	a.has_charge = (unsigned *)(sum + 2);
	a.part = sum + 4;
	char h_scr[256 * sizeof(int) + 4 * sizeof(double)];
	int *hfirst = (int *)h_scr;
	cudaError_t e = cudaMemsetAsync(scr, 0x7f, 256 * sizeof(int), d->st);   // "never seen"
	if (e == cudaSuccess) e = cudaMemsetAsync(sum, 0, 4 * sizeof(double), d->st);
	if (e == cudaSuccess) {
		a.pos = d->pos[0]; a.xn = d->xn; a.xlo = d->xlo;
		a.vhi = d->vhi; a.vlo = d->vlo; a.frc = d->frc;
		a.cross = d->cross; a.cbase = d->cbase;
		a.gid = d->gid; a.inv = d->inv; a.mol = d->mol; a.charge = d->charge;
		k_upload_parts<<<nb, HIO_B, 0, d->st>>>(a);
		k_upload_sum<<<1, 32, 0, d->st>>>(a.part, nb, sum);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaMemcpyAsync(h_scr, scr, sizeof h_scr, cudaMemcpyDeviceToHost, d->st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
	if (e != cudaSuccess) { sepdev_set_error("upload (in place)", e); rc = SEPDEV_ECUDA; }
	if (!rc) {
		// ids in order of first appearance, as the sequential host loop assigns them
		int order[256], k = 0;
		for (int c = 0; c < 256; c++)
			if (hfirst[c] >= 0 && hfirst[c] < n) order[k++] = c;
		for (int x = 1; x < k; x++)
			for (int y = x; y > 0 && hfirst[order[y]] < hfirst[order[y - 1]]; y--) {
				const int t = order[y]; order[y] = order[y - 1]; order[y - 1] = t;
			}
		if (k > max_types) { rc = SEPDEV_EOVERFLOW; sepdev_set_error("too many particle types", cudaErrorInvalidValue); }
		if (!rc) {
			TypeMap tm;
			for (int c = 0; c < 256; c++) tm.id[c] = 0;
			for (int t = 0; t < k; t++) { tm.id[order[t]] = t; tchar[t] = (char)order[t]; }
			*ntypes = k;
			k_upload_types<<<grid_for(n, 256), 256, 0, d->st>>>(n, d->pos[0], d->xn, tm);
			e = cudaGetLastError();
			if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
			if (e != cudaSuccess) { sepdev_set_error("upload (types)", e); rc = SEPDEV_ECUDA; }
		}
	}
	if (!rc) {
		const double *hs = (const double *)(h_scr + 256 * sizeof(int));
		*sumv2 = hs[0];
		unsigned long long mb;
		memcpy(&mb, &hs[1], sizeof mb);
		double md;
		memcpy(&md, &mb, sizeof md);
		*maxd2 = md;
		unsigned hc;
		memcpy(&hc, &hs[2], sizeof hc);
		d->has_charge = hc ? 1 : 0;
		d->cur = 0;
		d->list_valid = 0;
	}
	return rc;
}

struct HioDown {
	seppart *p;
	long n;
	double L[3];
	const int4 *pos, *cross, *cbase, *xn;
	const uint4 *xlo;
	const float4 *vhi, *vlo, *frc;
	const int *inv;
	int forces_zero;
	unsigned *bad;
};

// Words written back: x, v, f, a (head words 0-11), cross_neighb and
// crossings (the 24 bytes at their offset), xn.  One thread per record
// (user index order) fills its words in shared memory from the device arrays
// at its slot; the block then stores them as contiguous runs.
#define DW_XVFA 12
#define DW_CROSS 3
#define DW (DW_XVFA + DW_CROSS + HW_XN)
static_assert(offsetof(seppart, a) / 8 + 3 == DW_XVFA, "x v f a are words 0-11");
static_assert(offsetof(seppart, cross_neighb) % 8 == 0 &&
	      offsetof(seppart, crossings) == offsetof(seppart, cross_neighb) + 12, "crossing words");
#define CROSS_W (offsetof(seppart, cross_neighb) / 8)

__global__ void __launch_bounds__(HIO_B) k_download_parts(HioDown a)
{
	__shared__ unsigned long long sm[HIO_B][DW];
	const long r0 = blockIdx.x * (long)HIO_B;
	const int cnt = (int)min((long)HIO_B, a.n - r0);
	const long u = r0 + threadIdx.x;
	if (u < a.n) {
		const long s = a.inv[u];
		if (s < 0 || s >= a.n) atomicOr(a.bad, 1u);
		const long ss = (s < 0 || s >= a.n) ? 0 : s;
		const double m = a.p[u].m;
		const int4 ph = a.pos[ss];
		const uint4 pl = a.xlo[ss];
		const float4 vh = a.vhi[ss], vl = a.vlo[ss], f = a.frc[ss];
		const int4 c = a.cross[ss], cb = a.cbase[ss], xh = a.xn[ss];
		const unsigned hi[3] = {(unsigned)ph.x, (unsigned)ph.y, (unsigned)ph.z};
		const unsigned lo[3] = {pl.x, pl.y, pl.z};
		const float vhk[3] = {vh.x, vh.y, vh.z}, vlk[3] = {vl.x, vl.y, vl.z}, fk[3] = {f.x, f.y, f.z};
		const int ck[3] = {c.x, c.y, c.z}, cbk[3] = {cb.x, cb.y, cb.z};
		const unsigned xnk[3] = {(unsigned)xh.x, (unsigned)xh.y, (unsigned)xh.z};
		double *w = (double *)sm[threadIdx.x];
		int *wi = (int *)&sm[threadIdx.x][DW_XVFA];
		for (int k = 0; k < 3; k++) {
			w[k] = from_fixed_dev(hi[k], lo[k], a.L[k]);
			w[3 + k] = __dadd_rn((double)vhk[k], (double)vlk[k]);
			const double fd = a.forces_zero ? 0.0 : (double)fk[k];
			w[6 + k] = fd;
			w[9 + k] = __ddiv_rn(fd, m);
			wi[k] = ck[k] - cbk[k];          // cross_neighb
			wi[3 + k] = ck[k];               // crossings
			w[DW_XVFA + DW_CROSS + k] = from_fixed_dev(xnk[k], 0u, a.L[k]);
		}
	}
	__syncthreads();
	unsigned long long *g = (unsigned long long *)a.p;
	for (int q = threadIdx.x; q < cnt * DW; q += HIO_B) {
		const int r = q / DW, wq = q - r * DW;
		const long base = (r0 + r) * (long)RW;
		const long gi = wq < DW_XVFA ? base + wq
			      : (wq < DW_XVFA + DW_CROSS ? base + CROSS_W + wq - DW_XVFA
							  : base + XN_W + wq - DW_XVFA - DW_CROSS);
		g[gi] = sm[r][wq];
	}
}

extern "C" int sepdev_download_parts(sepdev *d, void *parts, int forces_zero)
{
	const long n = d->n;
	if (!d->hostio_direct) return SEPDEV_EINVAL;
	char *scr = NULL;
	int rc = hio_scratch(d, 256, &scr);
	if (rc) return rc;
	unsigned *bad = (unsigned *)scr;
	HioDown a;
	a.p = (seppart *)parts;
	a.n = n;
	for (int k = 0; k < 3; k++) a.L[k] = d->L[k];
	a.pos = d->pos[d->cur]; a.xlo = d->xlo; a.vhi = d->vhi; a.vlo = d->vlo; a.frc = d->frc;
	a.cross = d->cross; a.cbase = d->cbase; a.xn = d->xn; a.inv = d->inv;
	a.forces_zero = forces_zero;
	a.bad = bad;
	unsigned hbad = 0;
	cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(unsigned), d->st);
	if (e == cudaSuccess) {
		k_download_parts<<<grid_for(n, HIO_B), HIO_B, 0, d->st>>>(a);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaMemcpyAsync(&hbad, bad, sizeof hbad, cudaMemcpyDeviceToHost, d->st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
	if (e != cudaSuccess) { sepdev_set_error("download (in place)", e); return SEPDEV_ECUDA; }
	if (hbad) { sepdev_set_error("download: slot map corrupt", cudaErrorInvalidValue); return SEPDEV_EINVAL; }
	return SEPDEV_OK;
}
