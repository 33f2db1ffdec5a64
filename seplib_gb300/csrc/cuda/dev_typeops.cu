// dev_typeops.cu - operations on the particles of one type: the tether
// force towards x0 (reference source/sepmisc.c:645-670), the sums behind the
// temperature relaxation and the momentum reset (:357-391, :1173-1192) and
// the velocity update they apply, and the density / momentum / temperature
// profiles of the profs sampler (source/sepsampler.c:1453-1510).
//
// Sums are FP64 in a fixed order (per-block tree, blocks in order on the
// host); the profile histograms accumulate 64-bit fixed point (2^-32
// units), so their sums do not depend on the order of the atomics.
#include <math.h>
#include <stdlib.h>
#include "dev_common.cuh"

#define TB 256

static void *scratch(sepdev *d, size_t bytes)
{
	if (bytes > d->tscr_cap) {
		if (d->tscr) cudaFree(d->tscr);
		d->tscr = NULL;
		d->tscr_cap = 0;
		if (cudaMalloc(&d->tscr, bytes) != cudaSuccess) return NULL;
		d->tscr_cap = bytes;
	}
	return d->tscr;
}

// ---- tether force ------------------------------------------------------------

// f += k (x0 - x), the separation taken as the minimum image in FP64
__global__ void k_tether(long n, int tid, double k, const int4 *pos, const uint4 *xlo, const int *gid,
			 const double *x0, float4 *frc, double L0, double L1, double L2)
{
	const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
	if (i >= n) return;
	const int4 p = pos[i];
	if (p.w != tid) return;
	const uint4 l = xlo[i];
	const long u = gid[i];
	const double L[3] = {L0, L1, L2};
	const unsigned h[3] = {(unsigned)p.x, (unsigned)p.y, (unsigned)p.z}, lo[3] = {l.x, l.y, l.z};
	float g[3];
	for (int q = 0; q < 3; q++) {
		double r = x0[3 * u + q] - from_fixed_dev(h[q], lo[q], L[q]);
		if (r > 0.5 * L[q]) r -= L[q];
		else if (r < -0.5 * L[q]) r += L[q];
		g[q] = (float)(k * r);
	}
	float4 f = frc[i];
	f.x += g[0]; f.y += g[1]; f.z += g[2];
	frc[i] = f;
}

extern "C" int sepdev_set_x0(sepdev *d, const double *x0)
{
	if (!d->x0) CK(cudaMalloc((void **)&d->x0, sizeof(double) * 3 * d->n));
	CK(cudaMemcpyAsync(d->x0, x0, sizeof(double) * 3 * d->n, cudaMemcpyHostToDevice, d->st));
	CK(cudaStreamSynchronize(d->st));
	return SEPDEV_OK;
}

extern "C" int sepdev_tether(sepdev *d, int tid, double k)
{
	if (!d->x0) return SEPDEV_EINVAL;
	k_tether<<<grid_for(d->n, TB), TB, 0, d->st>>>(d->n, tid, k, d->pos[d->cur], d->xlo, d->gid, d->x0, d->frc,
							d->L[0], d->L[1], d->L[2]);
	CKL(d);
	return SEPDEV_OK;
}

// ---- per-type sums and velocity update ---------------------------------------

// per block: sum m v_k (3), sum m, sum m v^2, count over the particles of
// the type (v = hi + lo in FP64)
__global__ void __launch_bounds__(TB) k_type_sums(long n, int tid, const int4 *pos, const float4 *vhi,
						  const float4 *vlo, double *part)
{
	__shared__ double red[TB];
	const long i = blockIdx.x * (long)TB + threadIdx.x;
	double t[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
	if (i < n && pos[i].w == tid) {
		const float4 h = vhi[i], l = vlo[i];
		const double m = (double)h.w;
		const double v[3] = {(double)h.x + (double)l.x, (double)h.y + (double)l.y, (double)h.z + (double)l.z};
		for (int k = 0; k < 3; k++) {
			t[k] = m * v[k];
			t[4] += m * v[k] * v[k];
		}
		t[3] = m;
		t[5] = 1.0;
	}
	for (int q = 0; q < 6; q++) {
		red[threadIdx.x] = t[q];
		__syncthreads();
		for (int s = TB / 2; s > 0; s >>= 1) {
			if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
			__syncthreads();
		}
		if (threadIdx.x == 0) part[(long)blockIdx.x * 6 + q] = red[0];
		__syncthreads();
	}
}

extern "C" int sepdev_type_sums(sepdev *d, int tid, double *out)
{
	const int nblk = grid_for(d->n, TB);
	double *part = (double *)scratch(d, sizeof(double) * 6 * nblk);
	if (!part) { sepdev_set_error("type sums", cudaErrorMemoryAllocation); return SEPDEV_ENOMEM; }
	k_type_sums<<<nblk, TB, 0, d->st>>>(d->n, tid, d->pos[d->cur], d->vhi, d->vlo, part);
	CKL(d);
	double *h = (double *)malloc(sizeof(double) * 6 * nblk);
	if (!h) return SEPDEV_ENOMEM;
	cudaError_t e = cudaMemcpyAsync(h, part, sizeof(double) * 6 * nblk, cudaMemcpyDeviceToHost, d->st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
	if (e != cudaSuccess) { free(h); sepdev_set_error("type sums", e); return SEPDEV_ECUDA; }
	for (int q = 0; q < 6; q++) out[q] = 0.0;
	for (int b = 0; b < nblk; b++)
		for (int q = 0; q < 6; q++) out[q] += h[6 * b + q];
	free(h);
	return SEPDEV_OK;
}

// v = v fact - shift for the particles of the type, in FP64, stored back
// as the float pair (hi, lo)
__global__ void k_type_scale(long n, int tid, const int4 *pos, float4 *vhi, float4 *vlo, double fact, double s0,
			     double s1, double s2)
{
	const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
	if (i >= n || pos[i].w != tid) return;
	float4 h = vhi[i], l = vlo[i];
	const double sh[3] = {s0, s1, s2};
	float *hp[3] = {&h.x, &h.y, &h.z}, *lp[3] = {&l.x, &l.y, &l.z};
	for (int k = 0; k < 3; k++) {
		const double v = ((double)*hp[k] + (double)*lp[k]) * fact - sh[k];
		const float vh = (float)v;
		*hp[k] = vh;
		*lp[k] = (float)(v - (double)vh);
	}
	vhi[i] = h;
	vlo[i] = l;
}

extern "C" int sepdev_type_scale(sepdev *d, int tid, double fact, const double *shift)
{
	k_type_scale<<<grid_for(d->n, TB), TB, 0, d->st>>>(d->n, tid, d->pos[d->cur], d->vhi, d->vlo, fact, shift[0],
							    shift[1], shift[2]);
	CKL(d);
	return SEPDEV_OK;
}

// ---- profiles ------------------------------------------------------------------

// bins of width dl along dir; per bin (fixed point): sum m v[dirvel], sum m,
// sum m v^2 over the other two components, count
__global__ void __launch_bounds__(TB) k_profile(long n, int tid, int dir, int dirvel, int lvec, double L, double dl,
						const int4 *pos, const uint4 *xlo, const float4 *vhi, const float4 *vlo,
						unsigned long long *hist)
{
	extern __shared__ long long sh[];
	for (int k = threadIdx.x; k < 4 * lvec; k += blockDim.x) sh[k] = 0;
	__syncthreads();
	const long i = blockIdx.x * (long)TB + threadIdx.x;
	if (i < n) {
		const int4 p = pos[i];
		if (p.w == tid) {
			const uint4 l = xlo[i];
			const unsigned ph[3] = {(unsigned)p.x, (unsigned)p.y, (unsigned)p.z}, pl[3] = {l.x, l.y, l.z};
			int b = (int)(from_fixed_dev(ph[dir], pl[dir], L) / dl);
			b = b < 0 ? 0 : (b >= lvec ? lvec - 1 : b);
			const float4 h = vhi[i], lo = vlo[i];
			const double m = (double)h.w;
			const double v[3] = {(double)h.x + (double)lo.x, (double)h.y + (double)lo.y,
					     (double)h.z + (double)lo.z};
			double s2 = 0.0;
			for (int k = 0; k < 3; k++)
				if (k != dirvel) s2 += m * v[k] * v[k];
			atomicAdd((unsigned long long *)&sh[4 * b], (unsigned long long)llrint(ldexp(m * v[dirvel], 32)));
			atomicAdd((unsigned long long *)&sh[4 * b + 1], (unsigned long long)llrint(ldexp(m, 32)));
			atomicAdd((unsigned long long *)&sh[4 * b + 2], (unsigned long long)llrint(ldexp(s2, 32)));
			atomicAdd((unsigned long long *)&sh[4 * b + 3], 1ull);
		}
	}
	__syncthreads();
	for (int k = threadIdx.x; k < 4 * lvec; k += blockDim.x)
		if (sh[k]) atomicAdd(&hist[k], (unsigned long long)sh[k]);
}

extern "C" int sepdev_profile(sepdev *d, int tid, int dir, int dirvel, int lvec, double *out)
{
	if (dir < 0 || dir > 2 || dirvel < 0 || dirvel > 2 || lvec < 1 || 4 * (size_t)lvec * 8 > 48 * 1024)
		return SEPDEV_EINVAL;
	unsigned long long *hist = (unsigned long long *)scratch(d, sizeof(long long) * 4 * lvec);
	if (!hist) { sepdev_set_error("profile", cudaErrorMemoryAllocation); return SEPDEV_ENOMEM; }
	CK(cudaMemsetAsync(hist, 0, sizeof(long long) * 4 * lvec, d->st));
	const double L = d->L[dir];
	k_profile<<<grid_for(d->n, TB), TB, sizeof(long long) * 4 * lvec, d->st>>>(
		d->n, tid, dir, dirvel, lvec, L, L / lvec, d->pos[d->cur], d->xlo, d->vhi, d->vlo, hist);
	CKL(d);
	long long *h = (long long *)malloc(sizeof(long long) * 4 * lvec);
	if (!h) return SEPDEV_ENOMEM;
	cudaError_t e = cudaMemcpyAsync(h, hist, sizeof(long long) * 4 * lvec, cudaMemcpyDeviceToHost, d->st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
	if (e != cudaSuccess) { free(h); sepdev_set_error("profile", e); return SEPDEV_ECUDA; }
	for (int k = 0; k < 4 * lvec; k++) out[k] = (k % 4 == 3) ? (double)h[k] : ldexp((double)h[k], -32);
	free(h);
	return SEPDEV_OK;
}
