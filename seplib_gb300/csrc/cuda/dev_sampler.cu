// dev_sampler.cu - device parts of the vacf and msd samplers.
//
// The reference's samplers (source/sepsampler.c:471-714) read every
// particle's velocity or position on the host at each sample.  Here the
// data a sample needs never leaves the GPU:
//   vacf  the x-velocities of a block of lvec samples live in a device ring
//         indexed by user particle index; at the end of a block the
//         correlation C[k] = sum_i sum_kk v[kk][i] v[k + kk][i] is one
//         kernel (grid over lags and particles) plus an ordered sum;
//   msd   the reference positions (unwrapped, FP64) and the crossing counts
//         at the block start are kept per particle; a sample reduces
//         |dr|^2, |dr|^4 and cos(k dr_x) over the particles of one type on
//         the device and returns 2 + nk numbers.
// Reductions are FP64 with a fixed order (per-block tree, then blocks in
// order), so repeated runs give the same files.
#include <math.h>
#include <stdlib.h>
#include "dev_common.cuh"

#define SB 256

struct sepdev_vacf {
	double *ring;     // [lvec][n]
	double *part;     // [lvec][nblk] per-block partial sums
	double *sum;      // [lvec]
	long count;       // values per sample: particles, or molecules (mvacf)
	int lvec;
	int nblk;
};

struct sepdev_msd {
	double *pos0;     // [3 n] unwrapped positions at the block start
	int4 *cross0;     // [n] crossing counts at the block start
	double *kvec;     // [nk]
	double *part;     // [nblk][2 + nk]
	double *sum;      // [2 + nk]
	int nk;
	int nblk;
};

__device__ __forceinline__ double pos_dbl(unsigned hi, unsigned lo, double L)
{
	return __dmul_rn(__dadd_rn(ldexp((double)hi, -32), ldexp((double)lo, -64)), L);
}

// fixed-order tree over a block of SB threads; thread 0 returns the sum
__device__ __forceinline__ double block_sum_d(double v, double *red)
{
	red[threadIdx.x] = v;
	__syncthreads();
	for (int s = SB / 2; s > 0; s >>= 1) {
		if ((int)threadIdx.x < s) red[threadIdx.x] = __dadd_rn(red[threadIdx.x], red[threadIdx.x + s]);
		__syncthreads();
	}
	const double r = red[0];
	__syncthreads();
	return r;
}

// ---- vacf ----

__global__ void k_vacf_store(long n, const int *gid, const float4 *vhi, const float4 *vlo, double *row)
{
	const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
	if (t < n) row[gid[t]] = (double)vhi[t].x + (double)vlo[t].x;
}

// blockIdx.y = lag k; each thread sums its particle's products over kk
__global__ void __launch_bounds__(SB) k_vacf_lags(long n, int lvec, const double *ring, double *part)
{
	__shared__ double red[SB];
	const long i = blockIdx.x * (long)SB + threadIdx.x;
	const int k = blockIdx.y;
	double s = 0.0;
	if (i < n)
		for (int kk = 0; kk < lvec - k; kk++)
			s = __fma_rn(ring[(long)kk * n + i], ring[(long)(k + kk) * n + i], s);
	const double b = block_sum_d(s, red);
	if (threadIdx.x == 0) part[(long)k * gridDim.x + blockIdx.x] = b;
}

// one thread per row: ordered sum of nblk partials
__global__ void k_rows_sum(int rows, int nblk, const double *part, double *out, int row_major)
{
	const int r = blockIdx.x * blockDim.x + threadIdx.x;
	if (r >= rows) return;
	double s = 0.0;
	for (int b = 0; b < nblk; b++)
		s = __dadd_rn(s, row_major ? part[(long)r * nblk + b] : part[(long)b * rows + r]);
	out[r] = s;
}

extern "C" int sepdev_vacf_create_count(sepdev *d, int lvec, long count, sepdev_vacf **out)
{
	(void)d;
	*out = NULL;
	if (lvec < 1 || count < 1) return SEPDEV_EINVAL;
	sepdev_vacf *v = (sepdev_vacf *)calloc(1, sizeof *v);
	if (!v) return SEPDEV_ENOMEM;
	v->lvec = lvec;
	v->count = count;
	v->nblk = grid_for(count, SB);
	cudaError_t e = cudaMalloc((void **)&v->ring, sizeof(double) * lvec * count);
	if (e == cudaSuccess) e = cudaMalloc((void **)&v->part, sizeof(double) * lvec * v->nblk);
	if (e == cudaSuccess) e = cudaMalloc((void **)&v->sum, sizeof(double) * lvec);
	if (e != cudaSuccess) {
		cudaFree(v->ring); cudaFree(v->part); cudaFree(v->sum); free(v);
		sepdev_set_error("vacf buffers", e);
		return SEPDEV_ENOMEM;
	}
	*out = v;
	return SEPDEV_OK;
}

extern "C" int sepdev_vacf_create(sepdev *d, int lvec, sepdev_vacf **out)
{
	return sepdev_vacf_create_count(d, lvec, d->n, out);
}

double *sepdev_vacf_row(sepdev_vacf *v, int index)
{
	if (index < 0 || index >= v->lvec) return NULL;
	return v->ring + (long)index * v->count;
}

long sepdev_vacf_count(const sepdev_vacf *v) { return v->count; }

extern "C" void sepdev_vacf_destroy(sepdev_vacf *v)
{
	if (!v) return;
	cudaFree(v->ring); cudaFree(v->part); cudaFree(v->sum);
	free(v);
}

extern "C" int sepdev_vacf_store(sepdev *d, sepdev_vacf *v, int index)
{
	if (index < 0 || index >= v->lvec || v->count != d->n) return SEPDEV_EINVAL;
	k_vacf_store<<<grid_for(d->n, SB), SB, 0, d->st>>>(d->n, d->gid, d->vhi, d->vlo, v->ring + (long)index * d->n);
	CKL(d);
	return SEPDEV_OK;
}

// C[k] of the block in the ring, k = 0 .. lvec-1, into out (host)
extern "C" int sepdev_vacf_block(sepdev *d, sepdev_vacf *v, double *out)
{
	dim3 grid(v->nblk, v->lvec);
	k_vacf_lags<<<grid, SB, 0, d->st>>>(v->count, v->lvec, v->ring, v->part);
	k_rows_sum<<<grid_for(v->lvec, 128), 128, 0, d->st>>>(v->lvec, v->nblk, v->part, v->sum, 1);
	CKL(d);
	CK(cudaMemcpyAsync(out, v->sum, sizeof(double) * v->lvec, cudaMemcpyDeviceToHost, d->st));
	CK(cudaStreamSynchronize(d->st));
	return SEPDEV_OK;
}

// ---- msd ----

struct MsdArgs {
	long n;
	double L[3];
	const int4 *pos;
	const uint4 *xlo;
	const int4 *cross;
	const int *gid;
	double *pos0;
	int4 *cross0;
	const double *kvec;
	int nk;
	int type_id;
	double *part;
};

__global__ void k_msd_base(MsdArgs a)
{
	const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
	if (t >= a.n) return;
	const long u = a.gid[t];
	const int4 p = a.pos[t];
	const uint4 l = a.xlo[t];
	a.pos0[3 * u] = pos_dbl((unsigned)p.x, l.x, a.L[0]);
	a.pos0[3 * u + 1] = pos_dbl((unsigned)p.y, l.y, a.L[1]);
	a.pos0[3 * u + 2] = pos_dbl((unsigned)p.z, l.z, a.L[2]);
	a.cross0[u] = a.cross[t];
}

// per block: sum of |dr|^2, |dr|^4, cos(k_j dr_x) over the particles of the type
__global__ void __launch_bounds__(SB) k_msd_sample(MsdArgs a)
{
	__shared__ double red[SB];
	const long t = blockIdx.x * (long)SB + threadIdx.x;
	const int m = 2 + a.nk;
	bool on = false;
	double dr[3] = {0.0, 0.0, 0.0};
	if (t < a.n) {
		const int4 p = a.pos[t];
		if (p.w == a.type_id) {
			on = true;
			const long u = a.gid[t];
			const uint4 l = a.xlo[t];
			const int4 c = a.cross[t], c0 = a.cross0[u];
			const unsigned hi[3] = {(unsigned)p.x, (unsigned)p.y, (unsigned)p.z};
			const unsigned lo[3] = {l.x, l.y, l.z};
			const int dc[3] = {c.x - c0.x, c.y - c0.y, c.z - c0.z};
			for (int k = 0; k < 3; k++)
				dr[k] = __dsub_rn(__dadd_rn(pos_dbl(hi[k], lo[k], a.L[k]), __dmul_rn((double)dc[k], a.L[k])),
						  a.pos0[3 * u + k]);
		}
	}
	const double sq = on ? __dadd_rn(__dadd_rn(__dmul_rn(dr[0], dr[0]), __dmul_rn(dr[1], dr[1])),
				       __dmul_rn(dr[2], dr[2])) : 0.0;
	for (int j = 0; j < m; j++) {
		double v = 0.0;
		if (on) v = j == 0 ? sq : (j == 1 ? __dmul_rn(sq, sq) : cos(a.kvec[j - 2] * dr[0]));
		const double b = block_sum_d(v, red);
		if (threadIdx.x == 0) a.part[(long)blockIdx.x * m + j] = b;
	}
}

extern "C" int sepdev_msd_create(sepdev *d, int nk, const double *k, sepdev_msd **out)
{
	*out = NULL;
	if (nk < 0) return SEPDEV_EINVAL;
	sepdev_msd *m = (sepdev_msd *)calloc(1, sizeof *m);
	if (!m) return SEPDEV_ENOMEM;
	m->nk = nk;
	m->nblk = grid_for(d->n, SB);
	cudaError_t e = cudaMalloc((void **)&m->pos0, sizeof(double) * 3 * d->n);
	if (e == cudaSuccess) e = cudaMalloc((void **)&m->cross0, sizeof(int4) * d->n);
	if (e == cudaSuccess) e = cudaMalloc((void **)&m->kvec, sizeof(double) * (nk > 0 ? nk : 1));
	if (e == cudaSuccess) e = cudaMalloc((void **)&m->part, sizeof(double) * (2 + nk) * m->nblk);
	if (e == cudaSuccess) e = cudaMalloc((void **)&m->sum, sizeof(double) * (2 + nk));
	if (e == cudaSuccess && nk > 0) e = cudaMemcpy(m->kvec, k, sizeof(double) * nk, cudaMemcpyHostToDevice);
	if (e != cudaSuccess) {
		cudaFree(m->pos0); cudaFree(m->cross0); cudaFree(m->kvec); cudaFree(m->part); cudaFree(m->sum);
		free(m);
		sepdev_set_error("msd buffers", e);
		return SEPDEV_ENOMEM;
	}
	*out = m;
	return SEPDEV_OK;
}

extern "C" void sepdev_msd_destroy(sepdev_msd *m)
{
	if (!m) return;
	cudaFree(m->pos0); cudaFree(m->cross0); cudaFree(m->kvec); cudaFree(m->part); cudaFree(m->sum);
	free(m);
}

static MsdArgs msd_args(sepdev *d, sepdev_msd *m, int type_id)
{
	MsdArgs a;
	a.n = d->n;
	for (int k = 0; k < 3; k++) a.L[k] = d->L[k];
	a.pos = d->pos[d->cur];
	a.xlo = d->xlo;
	a.cross = d->cross;
	a.gid = d->gid;
	a.pos0 = m->pos0;
	a.cross0 = m->cross0;
	a.kvec = m->kvec;
	a.nk = m->nk;
	a.type_id = type_id;
	a.part = m->part;
	return a;
}

// the current positions become the block's reference
extern "C" int sepdev_msd_base(sepdev *d, sepdev_msd *m)
{
	k_msd_base<<<grid_for(d->n, SB), SB, 0, d->st>>>(msd_args(d, m, -1));
	CKL(d);
	return SEPDEV_OK;
}

// out (host, 2 + nk): sum |dr|^2, sum |dr|^4, sum cos(k_j dr_x) over type type_id
extern "C" int sepdev_msd_sample(sepdev *d, sepdev_msd *m, int type_id, double *out)
{
	const int cols = 2 + m->nk;
	k_msd_sample<<<m->nblk, SB, 0, d->st>>>(msd_args(d, m, type_id));
	k_rows_sum<<<grid_for(cols, 128), 128, 0, d->st>>>(cols, m->nblk, m->part, m->sum, 0);
	CKL(d);
	CK(cudaMemcpyAsync(out, m->sum, sizeof(double) * cols, cudaMemcpyDeviceToHost, d->st));
	CK(cudaStreamSynchronize(d->st));
	return SEPDEV_OK;
}

// ---- radial distribution (source/sepsampler.c:396-461) -------------------------
//
// Every pair i < j within half the box: bin floor(r / dg), one count for
// each requested type combination the pair matches.  The bin is found in
// FP32 from the exact fixed-point differences; a pair whose r / dg lies
// within RAD_EPS of a bin edge is recomputed with the reference's own FP64
// operations (positions as doubles, sep_Wrap by L_x on every axis, the
// squares summed in order, correctly rounded sqrt and division), so the
// counts are the reference's exactly.  A non-cubic box takes the FP64 path
// for every pair.  Blocks keep 32-bit counts in shared memory and add them
// to the 64-bit global histogram once.

#define RAD_B 256
#define RAD_G 16           // j tiles per block
#define RAD_EPS 1e-3f

struct RadArgs {
	long n;
	int lvec, ncomb, nt;
	double L, dg;          // the reference's lbox = L_x and bin width
	float fsx, fsy, fsz;   // L_k / 2^32
	float idg;             // 1 / dg
	int cubic;
	const int4 *pos;
	const uint4 *xlo;
	const unsigned *mask;  // [type i][type j] -> bit c: combination c matches
	unsigned long long *hist;   // [lvec][ncomb]
};

__device__ __forceinline__ int rad_bin64(const RadArgs &a, int4 pi, uint4 li, int4 pj, uint4 lj, double Ly, double Lz)
{
	const unsigned hi[3] = {(unsigned)pi.x, (unsigned)pi.y, (unsigned)pi.z};
	const unsigned lo[3] = {li.x, li.y, li.z};
	const unsigned hj[3] = {(unsigned)pj.x, (unsigned)pj.y, (unsigned)pj.z};
	const unsigned lj_[3] = {lj.x, lj.y, lj.z};
	const double Lk[3] = {a.L, Ly, Lz};
	double r2 = 0.0;
	for (int k = 0; k < 3; k++) {
		double rv = __dsub_rn(from_fixed_dev(hi[k], lo[k], Lk[k]), from_fixed_dev(hj[k], lj_[k], Lk[k]));
		if (rv > 0.5 * a.L) rv = __dsub_rn(rv, a.L);
		else if (rv < -0.5 * a.L) rv = __dadd_rn(rv, a.L);
		r2 = __dadd_rn(r2, __dmul_rn(rv, rv));
	}
	return (int)__ddiv_rn(__dsqrt_rn(r2), a.dg);
}

__global__ void __launch_bounds__(RAD_B) k_radial(RadArgs a, double Ly, double Lz)
{
	extern __shared__ unsigned char rsh[];
	int4 *sp = (int4 *)rsh;
	uint4 *sl = (uint4 *)(rsh + sizeof(int4) * RAD_B);
	unsigned *h = (unsigned *)(rsh + (sizeof(int4) + sizeof(uint4)) * RAD_B);
	const int nh = a.lvec * a.ncomb;
	for (int k = threadIdx.x; k < nh; k += RAD_B) h[k] = 0u;
	const int nb = (int)((a.n + RAD_B - 1) / RAD_B);
	const int bi = blockIdx.x;
	const int bj0 = max(bi, (int)blockIdx.y * RAD_G), bj1 = min(nb, ((int)blockIdx.y + 1) * RAD_G);
	const long i = (long)bi * RAD_B + threadIdx.x;
	const bool act = i < a.n;
	int4 pi = make_int4(0, 0, 0, 0);
	uint4 li = make_uint4(0, 0, 0, 0);
	if (act) { pi = a.pos[i]; li = a.xlo[i]; }
	const float lim = (float)a.lvec;
	__syncthreads();
	for (int bj = bj0; bj < bj1; bj++) {
		const long j0 = (long)bj * RAD_B;
		const long jl = j0 + threadIdx.x;
		if (jl < a.n) { sp[threadIdx.x] = a.pos[jl]; sl[threadIdx.x] = a.xlo[jl]; }
		__syncthreads();
		const int cnt = (int)min((long)RAD_B, a.n - j0);
		if (act) {
			const int k0 = bj == bi ? threadIdx.x + 1 : 0;
			for (int k = k0; k < cnt; k++) {
				const int4 pj = sp[k];
				int bin;
				if (a.cubic) {
					const float dx = (float)(int)((unsigned)pi.x - (unsigned)pj.x) * a.fsx;
					const float dy = (float)(int)((unsigned)pi.y - (unsigned)pj.y) * a.fsy;
					const float dz = (float)(int)((unsigned)pi.z - (unsigned)pj.z) * a.fsz;
					const float q = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) * a.idg;
					if (q > lim + 1.0f) continue;
					const float fl = floorf(q);
					if (q - fl < RAD_EPS || fl + 1.0f - q < RAD_EPS) bin = rad_bin64(a, pi, li, pj, sl[k], Ly, Lz);
					else bin = (int)fl;
				} else {
					bin = rad_bin64(a, pi, li, pj, sl[k], Ly, Lz);
				}
				if (bin >= a.lvec) continue;
				unsigned m = a.mask[pi.w * a.nt + pj.w];
				while (m) {
					const int c = __ffs(m) - 1;
					m &= m - 1;
					atomicAdd(&h[bin * a.ncomb + c], 1u);
				}
			}
		}
		__syncthreads();
	}
	for (int k = threadIdx.x; k < nh; k += RAD_B)
		if (h[k]) atomicAdd(&a.hist[k], (unsigned long long)h[k]);
}

// out (host, lvec x ncomb): the counts of one sample; mask[ti * nt + tj]
// (nt = the device's type count) holds the bits of the combinations the
// pair of type ids matches
extern "C" int sepdev_radial(sepdev *d, int lvec, int ncomb, int nt, const unsigned *mask, double *out)
{
	if (lvec < 1 || ncomb < 1 || ncomb > 32 || nt < 1 || nt > SEPDEV_MAXTYPES) return SEPDEV_EINVAL;
	const size_t hbytes = sizeof(unsigned) * lvec * ncomb;
	const size_t shm = (sizeof(int4) + sizeof(uint4)) * RAD_B + hbytes;
	if (shm > 200 * 1024) return SEPDEV_EINVAL;
	unsigned long long *hist = NULL;
	unsigned *dmask = NULL;
	cudaError_t e = cudaMalloc((void **)&hist, sizeof(unsigned long long) * lvec * ncomb);
	if (e == cudaSuccess) e = cudaMalloc((void **)&dmask, sizeof(unsigned) * nt * nt);
	if (e == cudaSuccess) e = cudaMemsetAsync(hist, 0, sizeof(unsigned long long) * lvec * ncomb, d->st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(dmask, mask, sizeof(unsigned) * nt * nt, cudaMemcpyHostToDevice, d->st);
	if (e == cudaSuccess && shm > 48 * 1024)
		e = cudaFuncSetAttribute(k_radial, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
	if (e != cudaSuccess) {
		cudaFree(hist); cudaFree(dmask);
		sepdev_set_error("radial distribution", e);
		return SEPDEV_ECUDA;
	}
	RadArgs a;
	a.n = d->n; a.lvec = lvec; a.ncomb = ncomb; a.nt = nt;
	a.L = d->L[0];
	a.dg = 0.5 * d->L[0] / lvec;
	a.fsx = d->fscale[0]; a.fsy = d->fscale[1]; a.fsz = d->fscale[2];
	a.idg = (float)(1.0 / a.dg);
	a.cubic = d->L[0] == d->L[1] && d->L[1] == d->L[2];
	a.pos = d->pos[d->cur]; a.xlo = d->xlo;
	a.mask = dmask; a.hist = hist;
	const int nb = grid_for(d->n, RAD_B);
	k_radial<<<dim3(nb, (nb + RAD_G - 1) / RAD_G), RAD_B, shm, d->st>>>(a, d->L[1], d->L[2]);
	CKL(d);
	unsigned long long *hh = (unsigned long long *)malloc(sizeof(unsigned long long) * lvec * ncomb);
	if (!hh) { cudaFree(hist); cudaFree(dmask); return SEPDEV_ENOMEM; }
	e = cudaMemcpyAsync(hh, hist, sizeof(unsigned long long) * lvec * ncomb, cudaMemcpyDeviceToHost, d->st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
	cudaFree(hist); cudaFree(dmask);
	if (e != cudaSuccess) { free(hh); sepdev_set_error("radial distribution", e); return SEPDEV_ECUDA; }
	for (int k = 0; k < lvec * ncomb; k++) out[k] = (double)hh[k];
	free(hh);
	return SEPDEV_OK;
}

// ---- atomic generalised hydrodynamics (source/sepsampler.c:957-1098) -----------
//
// Per wavevector k_j along y, over all particles, the sums of e^{i k_j y}
// (y unwrapped by the crossings, as the reference's xtrue) times m, m v_x,
// m v_y, the kinetic energy, 1, m a_y and m v_y^2; the reference's
// auxiliary sum m (a_y - i k v_y^2) e^{iky} is formed from the last two on
// the host.  FP64 with a fixed reduction order; nk x 14 numbers (plus the
// kinetic energy) come back per sample.

#define GH_N 15

struct sepdev_gh {
	double *kvec, *part, *sum;
	int nk, nblk;
};

__global__ void __launch_bounds__(SB) k_gh_sums(long n, double Ly, const int4 *pos, const uint4 *xlo,
						 const int4 *cross, const float4 *vhi, const float4 *vlo,
						 const float4 *frc, const double *kvec, double *part)
{
	__shared__ double red[SB / 32][GH_N];
	const long i = blockIdx.x * (long)SB + threadIdx.x;
	const int j = blockIdx.y;
	double t[GH_N];
	for (int q = 0; q < GH_N; q++) t[q] = 0.0;
	if (i < n) {
		const float4 h = vhi[i], l = vlo[i];
		const double m = (double)h.w;
		const double v[3] = {(double)h.x + (double)l.x, (double)h.y + (double)l.y, (double)h.z + (double)l.z};
		double ek = 0.0;
		for (int k = 0; k < 3; k++) ek += 0.5 * m * v[k] * v[k];
		const double y = Ly * cross[i].y + from_fixed_dev((unsigned)pos[i].y, xlo[i].y, Ly);
		double sn, cs;
		sincos(kvec[j] * y, &sn, &cs);
		const double ay = (double)frc[i].y / m;
		const double w[7] = {m, m * v[0], m * v[1], ek, 1.0, m * ay, m * v[1] * v[1]};
		for (int q = 0; q < 7; q++) {
			t[2 * q] = w[q] * cs;
			t[2 * q + 1] = w[q] * sn;
		}
		t[14] = ek;
	}
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	for (int q = 0; q < GH_N; q++) {
		double x = t[q];
		for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
		if (lane == 0) red[wid][q] = x;
	}
	__syncthreads();
	if (threadIdx.x < GH_N) {
		double x = 0.0;
		for (int w = 0; w < SB / 32; w++) x += red[w][threadIdx.x];
		part[((long)blockIdx.x * gridDim.y + j) * GH_N + threadIdx.x] = x;
	}
}

extern "C" int sepdev_gh_create(sepdev *d, int nk, const double *k, sepdev_gh **out)
{
	*out = NULL;
	if (nk < 1) return SEPDEV_EINVAL;
	sepdev_gh *g = (sepdev_gh *)calloc(1, sizeof *g);
	if (!g) return SEPDEV_ENOMEM;
	g->nk = nk;
	g->nblk = grid_for(d->n, SB);
	cudaError_t e = cudaMalloc((void **)&g->kvec, sizeof(double) * nk);
	if (e == cudaSuccess) e = cudaMalloc((void **)&g->part, sizeof(double) * GH_N * nk * g->nblk);
	if (e == cudaSuccess) e = cudaMalloc((void **)&g->sum, sizeof(double) * GH_N * nk);
	if (e == cudaSuccess) e = cudaMemcpy(g->kvec, k, sizeof(double) * nk, cudaMemcpyHostToDevice);
	if (e != cudaSuccess) {
		cudaFree(g->kvec); cudaFree(g->part); cudaFree(g->sum); free(g);
		sepdev_set_error("gh buffers", e);
		return SEPDEV_ENOMEM;
	}
	*out = g;
	return SEPDEV_OK;
}

extern "C" void sepdev_gh_destroy(sepdev_gh *g)
{
	if (!g) return;
	cudaFree(g->kvec); cudaFree(g->part); cudaFree(g->sum);
	free(g);
}

// out (host, 15 nk): for wavevector j, out[15 j + 2 q + (0 re, 1 im)] with q
// over (m, m v_x, m v_y, kinetic energy, 1, m a_y, m v_y^2) and
// out[15 j + 14] the sum of the kinetic energies
extern "C" int sepdev_gh_sample(sepdev *d, sepdev_gh *g, double *out)
{
	k_gh_sums<<<dim3(g->nblk, g->nk), SB, 0, d->st>>>(d->n, d->L[1], d->pos[d->cur], d->xlo, d->cross, d->vhi,
							  d->vlo, d->frc, g->kvec, g->part);
	// partials are [block][j][q]: row j * GH_N + q summed over the blocks in order
	k_rows_sum<<<grid_for(GH_N * g->nk, 128), 128, 0, d->st>>>(GH_N * g->nk, g->nblk, g->part, g->sum, 0);
	CKL(d);
	CK(cudaMemcpyAsync(out, g->sum, sizeof(double) * GH_N * g->nk, cudaMemcpyDeviceToHost, d->st));
	CK(cudaStreamSynchronize(d->st));
	return SEPDEV_OK;
}

// ---- partial coherent scattering (source/sepsampler.c:2142-2213) ----------------
//
// Per wavevector k_j = 2 pi (j + 1) / L_x and per requested type u (and, in
// the reference's 'i' mode, per molecule-index class: even, or odd or none)
// the sums of m e^{i k_j x} over the particles, x unwrapped by the
// crossings.  Warp shuffles and ordered block partials keep the FP64 sums
// independent of scheduling.

#define SC_MAXV 28     // 7 types x 2 classes x (re, im)

struct ScattArgs {
	long n;
	double Lx;
	const int4 *pos;
	const uint4 *xlo;
	const int4 *cross;
	const float4 *vhi;
	const int *mol;
	int umap[SEPDEV_MAXTYPES];     // device type id -> requested type index, -1
	int nu, nclass;                // requested types, classes (1: all; 2: even, odd-or-none)
	double *part;                  // [block][j][2 nu nclass]
};

__global__ void __launch_bounds__(SB) k_scatt(ScattArgs a)
{
	__shared__ double red[SB / 32][SC_MAXV];
	const long i = blockIdx.x * (long)SB + threadIdx.x;
	const int j = blockIdx.y;
	const int nv = 2 * a.nu * a.nclass;
	int u = -1, cls = 0;
	double re = 0.0, im = 0.0;
	if (i < a.n) {
		const int4 p = a.pos[i];
		u = a.umap[p.w];
		if (u >= 0) {
			const double m = (double)a.vhi[i].w;
			const double x = a.Lx * a.cross[i].x + from_fixed_dev((unsigned)p.x, a.xlo[i].x, a.Lx);
			const double k = 2.0 * 3.14159265358979 * (j + 1) / a.Lx;
			double sn, cs;
			sincos(k * x, &sn, &cs);
			re = m * cs;
			im = m * sn;
			const int mi = a.mol[i];
			// class bits: 1 = even molecule index, 2 = odd or no molecule
			cls = (mi >= 0 && mi % 2 == 0 ? 1 : 0) | ((mi + 1) % 2 == 0 ? 2 : 0);
		}
	}
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	for (int q = 0; q < nv; q++) {
		const int uq = q / (2 * a.nclass), cq = (q / 2) % a.nclass;
		const bool hit = u == uq && (a.nclass == 1 || (cls >> cq) & 1);
		double x = hit ? ((q & 1) ? im : re) : 0.0;
		for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
		if (lane == 0) red[wid][q] = x;
	}
	__syncthreads();
	if ((int)threadIdx.x < nv) {
		double x = 0.0;
		for (int w = 0; w < SB / 32; w++) x += red[w][threadIdx.x];
		a.part[((long)blockIdx.x * gridDim.y + j) * nv + threadIdx.x] = x;
	}
}

// umap (host, SEPDEV_MAXTYPES): requested type index of each device type id
// or -1; out (host, nk x 2 nu nclass): for wavevector j, type u, class c:
// out[j * 2 nu nclass + 2 (u nclass + c) + (0 re, 1 im)]
extern "C" int sepdev_scatt(sepdev *d, int nk, int nu, int nclass, const int *umap, double *out)
{
	if (nk < 1 || nu < 1 || (nclass != 1 && nclass != 2) || 2 * nu * nclass > SC_MAXV) return SEPDEV_EINVAL;
	const int nv = 2 * nu * nclass, nblk = grid_for(d->n, SB);
	double *part = NULL, *sum = NULL;
	cudaError_t e = cudaMalloc((void **)&part, sizeof(double) * nv * nk * nblk);
	if (e == cudaSuccess) e = cudaMalloc((void **)&sum, sizeof(double) * nv * nk);
	if (e != cudaSuccess) { cudaFree(part); sepdev_set_error("scatt buffers", e); return SEPDEV_ENOMEM; }
	ScattArgs a;
	a.n = d->n; a.Lx = d->L[0];
	a.pos = d->pos[d->cur]; a.xlo = d->xlo; a.cross = d->cross; a.vhi = d->vhi; a.mol = d->mol;
	for (int t = 0; t < SEPDEV_MAXTYPES; t++) a.umap[t] = umap[t];
	a.nu = nu; a.nclass = nclass; a.part = part;
	k_scatt<<<dim3(nblk, nk), SB, 0, d->st>>>(a);
	k_rows_sum<<<grid_for(nv * nk, 128), 128, 0, d->st>>>(nv * nk, nblk, part, sum, 0);
	CKL(d);
	e = cudaMemcpyAsync(out, sum, sizeof(double) * nv * nk, cudaMemcpyDeviceToHost, d->st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
	cudaFree(part); cudaFree(sum);
	if (e != cudaSuccess) { sepdev_set_error("scatt", e); return SEPDEV_ECUDA; }
	return SEPDEV_OK;
}
