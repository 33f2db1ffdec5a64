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
