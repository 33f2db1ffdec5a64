// dev_adj.cu - reverse-mode gradients through the LJ force and leap-frog
// (sepadj_* API), on the batched layout of dev_batch.cu.
//
// Forward (per replica, NVE): u_{n+1} = u_n + dt/m F(x_n), x_{n+1} = x_n +
// dt u_{n+1}, loss L = (1/K) sum_n l_n with l_n = U(x_n) + (sum m vt^2 +
// W(x_n)) / 3V, vt = (u_n + u_{n+1}) / 2, W = sum_pairs f.d.  Backward, with
// lx = dL/dx, lu = dL/du (zero after the last step), for n = K-1 .. 0:
//     g   = lu + dt lx + (1/K) m vt / 3V          (dL/du_{n+1} in total)
//     h   = dt/m g
//     lx += sum_j [ phi (h_i - h_j) + 2 phi' d (d.(h_i - h_j))
//                   + (2/K)(u' + w'/3V) d ]        (pair terms at x_n)
//     lu  = g + (1/K) m vt / 3V
// with per-pair functions of s = r^2: the force scalar phi (F_i = sum phi d,
// the reference's 48 eps s6 (s6 - aw/2) sigma^2/s), the energy u and the
// virial phi s; primes are d/ds.  The parameter gradients add, per pair and
// side, phi_theta d.h_i + (1/2K)(u_theta + phi_theta s / 3V).
//
// Slot order never changes after the initial sort: list rebuilds read the
// cells' members through index-only cell lists (the tile-staged build with
// an index indirection), so no permutation has to be undone in reverse.  Checkpoints every C steps hold the full replica state
// and list; the backward pass recomputes a segment from its checkpoint,
// keeping the states and the lists of every rebuilt replica, and sweeps it.
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <vector>
#include "dev_common.cuh"
#include "dev_batch.cuh"
#include "sepadj.h"
#include "sepbatch.h"

// ---- list rebuild without moving particles ----------------------------------

// a rebuilt system measures displacements from here on (skin test)
__global__ void ka_xn(const int *wsys, int nwarps, const unsigned *flag, const int4 *pos, int4 *xn,
		      const int4 *cross, int4 *cbase)
{
	const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
	const long wg = t >> 5;
	if (wg >= nwarps || !flag[wsys[wg]]) return;
	xn[t] = pos[t];
	cbase[t] = cross[t];
}

// ---- the backward step --------------------------------------------------------

struct AdjState {        // one stored step: positions and velocities per slot
	int4 *pos;
	uint4 *xlo;
	float4 *vhi, *vlo;
};

__device__ __forceinline__ double3 ff3(const float4 h, const float4 l)
{
	return make_double3((double)h.x + (double)l.x, (double)h.y + (double)l.y, (double)h.z + (double)l.z);
}

// g = lu + dt lx + kin, h = dt/m g, lu = g + kin  (kin = (1/K) m vt / 3V)
__global__ void ka_h(const BatchSys *sys, const int *wsys, int nwarps, AdjState un, AdjState un1,
		     double *lx, double *lu, float4 *h, double dt, double cK)
{
	const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
	const long wg = t >> 5;
	if (wg >= nwarps) return;
	const BatchSys S = sys[wsys[wg]];
	if (t - S.off >= S.n) {
		h[t] = make_float4(0.f, 0.f, 0.f, 0.f);
		return;
	}
	const float4 a0 = un.vhi[t], b0 = un.vlo[t], a1 = un1.vhi[t], b1 = un1.vlo[t];
	const double3 u0 = ff3(a0, b0), u1 = ff3(a1, b1);
	const double m = (double)a0.w;
	const double c = cK * m / (3.0 * S.L * S.L * S.L);
	const double vt[3] = {0.5 * (u0.x + u1.x), 0.5 * (u0.y + u1.y), 0.5 * (u0.z + u1.z)};
	double g[3];
	for (int k = 0; k < 3; k++) {
		const double kin = c * vt[k];
		g[k] = lu[3 * t + k] + dt * lx[3 * t + k] + kin;
		lu[3 * t + k] = g[k] + kin;
	}
	const double w = dt / m;
	h[t] = make_float4((float)(w * g[0]), (float)(w * g[1]), (float)(w * g[2]), 0.f);
}

// per type pair: the force parameters and what the gradient terms need
struct AdjPot {
	float rc2, sig2, eps48, eps4, aw, awh, ushift;
	float inv_eps, inv_sig, dsh_sig;   // 1/eps, 1/sigma, d ushift / d sigma
	int tu;                            // unordered type-pair index (gradient slot)
};

#define ADJ_MAXT SEPB_MAXTYPES

struct AdjPair {
	const BatchSys *sys;
	const int *wsys;
	int nwarps;
	const int4 *pos;         // x_n (high words; .w = type id)
	const int *pool;         // stored lists
	const long *lbase;       // per system: offset of its list at this step (ints)
	int maxnb;
	const float4 *h;
	double *lx;
	long long *gslots;       // per system: d/deps (NTP), then d/dsigma (NTP), fixed point
	const AdjPot *pot;       // NT x NT
	float cK;
};

// NT particle types, NTP = NT (NT + 1) / 2 type pairs, each with its own
// eps and sigma gradient
template <int NT>
__global__ void __launch_bounds__(256) ka_pair(AdjPair a)
{
	constexpr int NTP = NT * (NT + 1) / 2;
	__shared__ AdjPot sp[NT * NT];
	for (int k = threadIdx.x; k < NT * NT; k += blockDim.x) sp[k] = a.pot[k];
	__syncthreads();
	const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
	const long wg = i >> 5;
	if (wg >= a.nwarps) return;                   // whole warps
	const int sidx = a.wsys[wg];
	const BatchSys S = a.sys[sidx];
	const bool act = i - S.off < S.n;
	float lxx = 0.f, lxy = 0.f, lxz = 0.f, ge[NTP], gs[NTP];
#pragma unroll
	for (int t = 0; t < NTP; t++) { ge[t] = 0.f; gs[t] = 0.f; }
	if (act) {
		const float fs = S.fs;
		const float inv3V = (float)(1.0 / (3.0 * S.L * S.L * S.L));
		const int *lp = a.pool + a.lbase[sidx];
		const long li = i - S.off;                // index inside the system's list segment
		const int cnt = lp[(long)S.npad * a.maxnb + li];
		const int4 pi = a.pos[i];
		const float4 hi = a.h[i];
		const int row = NT > 1 ? pi.w * NT : 0;
		for (int k = 0; k < cnt; k++) {
			const int j = lp[nl_index(li, k, a.maxnb)];
			const int4 pj = a.pos[j];
			const AdjPot &pp = sp[NT > 1 ? row + pj.w : 0];
			const float dx = sep_hi(pi.x, pj.x, fs), dy = sep_hi(pi.y, pj.y, fs), dz = sep_hi(pi.z, pj.z, fs);
			const float s = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
			if (s >= pp.rc2) continue;
			const float is = 1.0f / s;
			const float q = pp.sig2 * is;
			const float s6 = q * q * q;
			const float phi = pp.eps48 * q * s6 * (s6 - pp.awh);
			const float phis = -pp.eps48 * q * s6 * (7.f * s6 - 4.f * pp.awh) * is;
			const float us = -0.25f * pp.eps48 * s6 * (2.f * s6 - pp.aw) * is;
			const float ws = -3.f * pp.eps48 * q * s6 * (2.f * s6 - pp.awh);
			const float u = pp.eps4 * s6 * (s6 - pp.aw) + pp.ushift;
			const float4 hj = a.h[j];
			const float dhx = hi.x - hj.x, dhy = hi.y - hj.y, dhz = hi.z - hj.z;
			const float ddh = dx * dhx + dy * dhy + dz * dhz;
			const float c2 = 2.f * phis * ddh + 2.f * a.cK * (us + ws * inv3V);
			lxx += phi * dhx + c2 * dx;
			lxy += phi * dhy + c2 * dy;
			lxz += phi * dhz + c2 * dz;
			const float dhi = dx * hi.x + dy * hi.y + dz * hi.z;
			const float phie = phi * pp.inv_eps, ue = u * pp.inv_eps;
			const float phisg = 2.f * pp.eps48 * q * s6 * (7.f * s6 - 4.f * pp.awh) * pp.inv_sig;
			const float usg = 0.5f * pp.eps48 * pp.inv_sig * s6 * (2.f * s6 - pp.aw) + pp.dsh_sig;
			const float te = phie * dhi + 0.5f * a.cK * (ue + phie * s * inv3V);
			const float ts = phisg * dhi + 0.5f * a.cK * (usg + phisg * s * inv3V);
#pragma unroll
			for (int t = 0; t < NTP; t++) {
				const bool mine = NTP == 1 || pp.tu == t;
				ge[t] += mine ? te : 0.f;
				gs[t] += mine ? ts : 0.f;
			}
		}
		a.lx[3 * i] += (double)lxx;
		a.lx[3 * i + 1] += (double)lxy;
		a.lx[3 * i + 2] += (double)lxz;
	}
	long long *g = a.gslots + 2 * NTP * (long)sidx;
#pragma unroll
	for (int t = 0; t < NTP; t++) {
		const long long qe = warp_sum_fx(to_fx(ge[t])), qs = warp_sum_fx(to_fx(gs[t]));
		if ((threadIdx.x & 31) == 0) {
			if (qe != 0) atomicAdd((unsigned long long *)&g[t], (unsigned long long)qe);
			if (qs != 0) atomicAdd((unsigned long long *)&g[NTP + t], (unsigned long long)qs);
		}
	}
}

// ---- host side ------------------------------------------------------------------

struct Ckpt {
	char *dev;                       // pos | xlo | vhi | vlo | xn | cross | cbase | ncnt | nl
	std::vector<BatchState> bs;
	std::vector<unsigned> flag;
	unsigned last_any;
	int cur;
};

struct sepadj {
	sepb *b;
	int C;
	long K;
	std::vector<Ckpt> ck;
	size_t ck_bytes;
	char *seg;                       // (C + 1) stored steps
	size_t seg_step_bytes;
	int *pool;
	long pool_cap, pool_used;
	std::vector<long> lbase;         // (C + 1) x nsys
	long *d_lbase;
	double *lx, *lu;
	float4 *h;
	long long *gslots;               // per replica: 2 NTP fixed-point gradients
	int nt, ntp;                     // particle types, type pairs
	AdjPot *dpot;                    // nt x nt
	unsigned *h_flag;                // pinned
	std::vector<double> loss;
	int have_forward;
	int at_end;                      // the device holds the state the last forward ended in
};

static size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

static void ck_layout(sepadj *A, size_t off[10])
{
	const long n = A->b->ntot;
	const int maxnb = A->b->d->maxnb;
	const size_t sz[9] = {16 * (size_t)n, 16 * (size_t)n, 16 * (size_t)n, 16 * (size_t)n,
			      16 * (size_t)n, 16 * (size_t)n, 16 * (size_t)n, 4 * (size_t)n,
			      4 * (size_t)n * maxnb};
	off[0] = 0;
	for (int k = 0; k < 9; k++) off[k + 1] = off[k] + al256(sz[k]);
}

static AdjState seg_state(sepadj *A, int k)
{
	const long n = A->b->ntot;
	char *p = A->seg + (size_t)k * A->seg_step_bytes;
	AdjState s;
	s.pos = (int4 *)p;
	s.xlo = (uint4 *)(p + al256(16 * (size_t)n));
	s.vhi = (float4 *)(p + 2 * al256(16 * (size_t)n));
	s.vlo = (float4 *)(p + 3 * al256(16 * (size_t)n));
	return s;
}

extern "C" void sepadj_destroy(sepadj *A)
{
	if (!A) return;
	if (A->b && A->b->d) cudaStreamSynchronize(A->b->d->st);
	for (auto &c : A->ck)
		if (c.dev) cudaFree(c.dev);
	void *dv[] = {A->seg, A->pool, A->d_lbase, A->lx, A->lu, A->h, A->gslots, A->dpot};
	for (size_t k = 0; k < sizeof dv / sizeof dv[0]; k++)
		if (dv[k]) cudaFree(dv[k]);
	if (A->h_flag) cudaFreeHost(A->h_flag);
	if (A->b) sepb_destroy(A->b);
	delete A;
}

// the per-type-pair table of the gradient kernel (params: nt x nt sets of
// {cf, eps, sigma, aw}; eps = 0: no term)
static int adj_pot_table(sepadj *A, int nt, const double *params)
{
	std::vector<AdjPot> t(nt * nt);
	for (int a = 0; a < nt; a++)
		for (int c = 0; c < nt; c++) {
			const double *p = params + 4 * (a * nt + c);
			AdjPot &q = t[a * nt + c];
			memset(&q, 0, sizeof q);
			const int lo = a < c ? a : c, hi = a < c ? c : a;
			q.tu = lo * nt - lo * (lo - 1) / 2 + (hi - lo);
			if (p[1] == 0.0) continue;           // rc2 = 0: the pair is skipped
			const double cf = p[0], eps = p[1], sig = p[2], aw = p[3];
			const double sr6 = pow(sig / cf, 6.0);
			q.rc2 = (float)(cf * cf);
			q.sig2 = (float)(sig * sig);
			q.eps48 = (float)(48.0 * eps);
			q.eps4 = (float)(4.0 * eps);
			q.aw = (float)aw;
			q.awh = (float)(0.5 * aw);
			q.ushift = (float)(-4.0 * eps * (sr6 * sr6 - aw * sr6));
			q.inv_eps = (float)(1.0 / eps);
			q.inv_sig = (float)(1.0 / sig);
			q.dsh_sig = (float)(-24.0 * eps / sig * (2.0 * sr6 * sr6 - aw * sr6));
		}
	A->nt = nt;
	A->ntp = nt * (nt + 1) / 2;
	CK(cudaMalloc((void **)&A->dpot, sizeof(AdjPot) * nt * nt));
	CK(cudaMemcpy(A->dpot, t.data(), sizeof(AdjPot) * nt * nt, cudaMemcpyHostToDevice));
	return SEPDEV_OK;
}

static sepadj *adj_make(sepb *b, int nrep, int nt, const double *params, int ckpt_every)
{
	if (!b) return NULL;
	sepadj *A = new sepadj();
	A->b = b;
	A->C = ckpt_every;
	const long n = b->ntot;
	if (adj_pot_table(A, nt, params)) {
		sepadj_destroy(A);
		return NULL;
	}
	cudaError_t e = cudaMalloc((void **)&A->lx, sizeof(double) * 3 * n);
	if (e == cudaSuccess) e = cudaMalloc((void **)&A->lu, sizeof(double) * 3 * n);
	if (e == cudaSuccess) e = cudaMalloc((void **)&A->h, sizeof(float4) * n);
	if (e == cudaSuccess) e = cudaMalloc((void **)&A->gslots, sizeof(long long) * 2 * A->ntp * nrep);
	if (e == cudaSuccess) e = cudaMallocHost((void **)&A->h_flag, sizeof(unsigned) * nrep);
	if (e != cudaSuccess) {
		sepdev_set_error("sepadj_create", e);
		sepadj_destroy(A);
		return NULL;
	}
	A->loss.assign(nrep, 0.0);
	return A;
}

extern "C" sepadj *sepadj_create(int nrep, const int *npart, const double *L, double rc, double skin,
				 double dt, const double *ljparam, int ckpt_every)
{
	if (!ljparam || ckpt_every < 1) {
		batch_fail("sepadj_create: ljparam and ckpt_every >= 1 are required", SEPDEV_EINVAL);
		return NULL;
	}
	return adj_make(sepb_create(nrep, npart, L, rc, skin, dt, ljparam), nrep, 1, ljparam, ckpt_every);
}

extern "C" sepadj *sepadj_create_typed(int nrep, const int *npart, const double *L, double skin, double dt,
				       int ntypes, const double *ljparams, int ckpt_every)
{
	if (!ljparams || ckpt_every < 1 || ntypes < 1 || ntypes > ADJ_MAXT) {
		batch_fail("sepadj_create_typed: 1 to 4 types, their parameters and ckpt_every >= 1 are required",
			   SEPDEV_EINVAL);
		return NULL;
	}
	return adj_make(sepb_create_typed(nrep, npart, L, skin, dt, ntypes, ljparams), nrep, ntypes, ljparams,
			ckpt_every);
}

extern "C" int sepadj_set_state(sepadj *A, int r, const double *x, const double *v, const double *m)
{
	if (!A) return batch_fail("sepadj_set_state: no adjoint", SEPDEV_EINVAL);
	A->have_forward = 0;
	for (auto &c : A->ck) { if (c.dev) cudaFree(c.dev); c.dev = NULL; }
	A->ck.clear();
	return sepb_set_state(A->b, r, x, v, m);
}

extern "C" int sepadj_set_types(sepadj *A, int r, const int *type)
{
	if (!A) return batch_fail("sepadj_set_types: no adjoint", SEPDEV_EINVAL);
	A->have_forward = 0;
	for (auto &c : A->ck) { if (c.dev) cudaFree(c.dev); c.dev = NULL; }
	A->ck.clear();
	return sepb_set_types(A->b, r, type);
}

// sort-free list rebuild of the flagged systems from buffer `parity`
static int adj_rebuild(sepadj *A, int parity)
{
	sepb *b = A->b;
	sepdev *d = b->d;
	int rc = batch_cells_launch(b, parity);
	if (rc) return rc;
	CK(cudaMemsetAsync(d->flags, 0, sizeof(unsigned) * 2, d->st));
	// the tile-staged build of the batched systems, reading each cell's
	// members through the index-only cell lists
	if ((rc = sepdev_batch_build(d, parity, b->cellstart, b->sys, b->wsys, b->nwarps, b->flag,
				     (float)((b->rc + b->skin) * (b->rc + b->skin)), d->perm)))
		return rc;
	ka_xn<<<grid_for(b->ntot, 256), 256, 0, d->st>>>(b->wsys, b->nwarps, b->flag, d->pos[parity], d->xn,
							d->cross, d->cbase);
	CKL(d);
	return SEPDEV_OK;
}

static int ck_save(sepadj *A, Ckpt &c)
{
	sepb *b = A->b;
	sepdev *d = b->d;
	const long n = b->ntot;
	size_t off[10];
	ck_layout(A, off);
	if (!c.dev) CK(cudaMalloc((void **)&c.dev, off[9]));
	char *p = c.dev;
	CK(cudaMemcpyAsync(p + off[0], d->pos[d->cur], 16 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(p + off[1], d->xlo, 16 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(p + off[2], d->vhi, 16 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(p + off[3], d->vlo, 16 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(p + off[4], d->xn, 16 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(p + off[5], d->cross, 16 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(p + off[6], d->cbase, 16 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(p + off[7], d->ncnt, 4 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(p + off[8], d->nl, 4 * (size_t)n * d->maxnb, cudaMemcpyDeviceToDevice, d->st));
	c.bs.resize(b->nsys);
	c.flag.resize(b->nsys);
	CK(cudaMemcpyAsync(c.bs.data(), b->bs, sizeof(BatchState) * b->nsys, cudaMemcpyDeviceToHost, d->st));
	CK(cudaMemcpyAsync(c.flag.data(), b->flag, sizeof(unsigned) * b->nsys, cudaMemcpyDeviceToHost, d->st));
	CK(cudaStreamSynchronize(d->st));
	c.last_any = b->h_run->last_any;
	c.cur = d->cur;
	return SEPDEV_OK;
}

static int ck_restore(sepadj *A, const Ckpt &c)
{
	sepb *b = A->b;
	sepdev *d = b->d;
	const long n = b->ntot;
	size_t off[10];
	ck_layout(A, off);
	d->cur = c.cur;
	const char *p = c.dev;
	CK(cudaMemcpyAsync(d->pos[d->cur], p + off[0], 16 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(d->xlo, p + off[1], 16 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(d->vhi, p + off[2], 16 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(d->vlo, p + off[3], 16 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(d->xn, p + off[4], 16 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(d->cross, p + off[5], 16 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(d->cbase, p + off[6], 16 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(d->ncnt, p + off[7], 4 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(d->nl, p + off[8], 4 * (size_t)n * d->maxnb, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(b->bs, c.bs.data(), sizeof(BatchState) * b->nsys, cudaMemcpyHostToDevice, d->st));
	CK(cudaMemcpyAsync(b->flag, c.flag.data(), sizeof(unsigned) * b->nsys, cudaMemcpyHostToDevice, d->st));
	b->h_run->last_any = c.last_any;
	CK(cudaStreamSynchronize(d->st));
	return SEPDEV_OK;
}

// one NVE step of every replica from the host (fused step, decision); the
// caller rebuilds first when the last decision asked for it.  Leaves the
// flags of the new decision in h_flag.
static int adj_step(sepadj *A, double loss_scale)
{
	sepb *b = A->b;
	sepdev *d = b->d;
	BatchRun *h = b->h_run;
	int rc;
	BatchDecide dec = batch_decide_args(b);
	dec.loss_scale = loss_scale;
	const long done0 = h->done;
	if ((rc = batch_step_launch(b, d->cur, dec))) return rc;
	CK(cudaMemcpyAsync(h, b->run, sizeof *h, cudaMemcpyDeviceToHost, d->st));
	CK(cudaMemcpyAsync(A->h_flag, b->flag, sizeof(unsigned) * b->nsys, cudaMemcpyDeviceToHost, d->st));
	CK(cudaStreamSynchronize(d->st));
	if ((h->done - done0) & 1) d->cur ^= 1;
	if (h->abort) return batch_fail("sepadj: neighbour list overflow", SEPDEV_EOVERFLOW);
	return SEPDEV_OK;
}

static int run_reset(sepadj *A)
{
	sepb *b = A->b;
	sepdev *d = b->d;
	BatchRun &r = *b->h_run;
	const unsigned la = r.last_any;
	memset(&r, 0, sizeof r);
	r.total = 0;                     // every step reports its observables
	r.last_any = la;
	CK(cudaMemcpyAsync(b->run, &r, sizeof r, cudaMemcpyHostToDevice, d->st));
	CK(cudaMemsetAsync(b->slots, 0, sizeof(long long) * SLOT_FIELDS * b->nsys, d->st));
	CK(cudaMemsetAsync(d->flags, 0, sizeof(unsigned) * 2, d->st));
	return SEPDEV_OK;
}

extern "C" int sepadj_forward(sepadj *A, long nsteps, double *loss)
{
	if (!A || nsteps < 1) return batch_fail("sepadj_forward: invalid arguments", SEPDEV_EINVAL);
	sepb *b = A->b;
	int rc;
	for (int s = 0; s < b->nsys; s++)
		if (!b->have[s]) return batch_fail("sepadj_forward: a replica has no state", SEPDEV_EINVAL);
	const long nseg = (nsteps + A->C - 1) / A->C;
	if (A->ck.empty()) {
		// the initial lists (sorted once) and the initial state
		if ((rc = batch_initial_lists(b))) return rc;
		b->h_run->last_any = 0;
		CK(cudaMemcpy(b->bs, b->h_bs, sizeof(BatchState) * b->nsys, cudaMemcpyHostToDevice));
		A->ck.resize(1);
		if ((rc = ck_save(A, A->ck[0]))) return rc;
	} else if ((rc = ck_restore(A, A->ck[0]))) {
		return rc;
	}
	if ((long)A->ck.size() < nseg) A->ck.resize(nseg);
	// loss accumulators start at zero
	std::vector<BatchState> bs(b->nsys);
	CK(cudaMemcpy(bs.data(), b->bs, sizeof(BatchState) * b->nsys, cudaMemcpyDeviceToHost));
	for (auto &x : bs) x.loss = 0.0;
	CK(cudaMemcpy(b->bs, bs.data(), sizeof(BatchState) * b->nsys, cudaMemcpyHostToDevice));
	if ((rc = run_reset(A))) return rc;
	const double cK = 1.0 / (double)nsteps;
	for (long n = 0; n < nsteps; n++) {
		if (n % A->C == 0 && n > 0 && (rc = ck_save(A, A->ck[n / A->C]))) return rc;
		if (b->h_run->last_any && (rc = adj_rebuild(A, b->d->cur))) return rc;
		if ((rc = adj_step(A, cK))) return rc;
	}
	CK(cudaMemcpy(bs.data(), b->bs, sizeof(BatchState) * b->nsys, cudaMemcpyDeviceToHost));
	for (int s = 0; s < b->nsys; s++) {
		A->loss[s] = bs[s].loss;
		if (loss) loss[s] = bs[s].loss;
	}
	A->K = nsteps;
	A->have_forward = 1;
	A->at_end = 1;
	return SEPDEV_OK;
}

static int seg_alloc(sepadj *A)
{
	sepb *b = A->b;
	const long n = b->ntot;
	const int maxnb = b->d->maxnb;
	A->seg_step_bytes = 4 * al256(16 * (size_t)n);
	if (!A->seg) CK(cudaMalloc((void **)&A->seg, A->seg_step_bytes * (A->C + 1)));
	// every system may be rebuilt at every step of a segment
	const long per_step = (long)n * maxnb + n;
	if (!A->pool) {
		A->pool_cap = per_step * (A->C + 2);
		CK(cudaMalloc((void **)&A->pool, sizeof(int) * A->pool_cap));
	}
	if (!A->d_lbase) CK(cudaMalloc((void **)&A->d_lbase, sizeof(long) * b->nsys * (A->C + 1)));
	A->lbase.assign((size_t)b->nsys * (A->C + 1), 0);
	return SEPDEV_OK;
}

// copy system s's current list (and counts) into the pool; returns its offset
static int snap(sepadj *A, int s, long *where)
{
	sepb *b = A->b;
	sepdev *d = b->d;
	const BatchSys &S = b->hsys[s];
	const long len = (long)S.npad * d->maxnb;
	if (A->pool_used + len + S.npad > A->pool_cap) return batch_fail("sepadj: list pool full", SEPDEV_ENOMEM);
	*where = A->pool_used;
	CK(cudaMemcpyAsync(A->pool + A->pool_used, d->nl + (long)S.off * d->maxnb, sizeof(int) * len,
			   cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(A->pool + A->pool_used + len, d->ncnt + S.off, sizeof(int) * S.npad,
			   cudaMemcpyDeviceToDevice, d->st));
	A->pool_used += len + S.npad;
	return SEPDEV_OK;
}

static int seg_store(sepadj *A, int k)
{
	sepdev *d = A->b->d;
	const long n = A->b->ntot;
	AdjState s = seg_state(A, k);
	CK(cudaMemcpyAsync(s.pos, d->pos[d->cur], 16 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(s.xlo, d->xlo, 16 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(s.vhi, d->vhi, 16 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	CK(cudaMemcpyAsync(s.vlo, d->vlo, 16 * (size_t)n, cudaMemcpyDeviceToDevice, d->st));
	return SEPDEV_OK;
}

static int adj_backward(sepadj *A, double *dloss_deps, double *dloss_dsigma, double *dloss_dx0)
{
	if (!A || !A->have_forward) return batch_fail("sepadj_backward: no forward pass", SEPDEV_EINVAL);
	sepb *b = A->b;
	sepdev *d = b->d;
	const long n = b->ntot;
	const int nsys = b->nsys;
	int rc;
	if ((rc = seg_alloc(A))) return rc;
	CK(cudaMemsetAsync(A->lx, 0, sizeof(double) * 3 * n, d->st));
	CK(cudaMemsetAsync(A->lu, 0, sizeof(double) * 3 * n, d->st));
	const int ntp = A->ntp;
	A->at_end = 0;
	CK(cudaMemsetAsync(A->gslots, 0, sizeof(long long) * 2 * ntp * nsys, d->st));
	const double cK = 1.0 / (double)A->K;
	AdjPair P;
	memset(&P, 0, sizeof P);
	P.sys = b->sys; P.wsys = b->wsys; P.nwarps = b->nwarps; P.pool = A->pool;
	P.maxnb = d->maxnb; P.h = A->h; P.lx = A->lx; P.gslots = A->gslots;
	P.pot = A->dpot;
	P.cK = (float)cK;
	const long nseg = (A->K + A->C - 1) / A->C;
	for (long sg = nseg - 1; sg >= 0; sg--) {
		const long c0 = sg * A->C, c1 = c0 + A->C < A->K ? c0 + A->C : A->K;
		const int m = (int)(c1 - c0);
		// recompute the segment from its checkpoint, keeping states and lists
		if ((rc = ck_restore(A, A->ck[sg]))) return rc;
		if ((rc = run_reset(A))) return rc;
		A->pool_used = 0;
		for (int s = 0; s < nsys; s++)
			if ((rc = snap(A, s, &A->lbase[s]))) return rc;
		memcpy(A->h_flag, A->ck[sg].flag.data(), sizeof(unsigned) * nsys);
		for (int k = 0; k < m; k++) {
			if ((rc = seg_store(A, k))) return rc;
			long *lb = &A->lbase[(size_t)k * nsys];
			if (k > 0) memcpy(lb, lb - nsys, sizeof(long) * nsys);
			const bool rebuild = b->h_run->last_any != 0;
			std::vector<unsigned> fl(A->h_flag, A->h_flag + nsys);
			if (rebuild && (rc = adj_rebuild(A, d->cur))) return rc;
			if (rebuild)
				for (int s = 0; s < nsys; s++)
					if (fl[s] && (rc = snap(A, s, &lb[s]))) return rc;
			if ((rc = adj_step(A, 0.0))) return rc;
		}
		if ((rc = seg_store(A, m))) return rc;
		CK(cudaMemcpyAsync(A->d_lbase, A->lbase.data(), sizeof(long) * nsys * m, cudaMemcpyHostToDevice,
				   d->st));
		// the backward sweep of the segment
		for (int k = m - 1; k >= 0; k--) {
			ka_h<<<grid_for(n, 256), 256, 0, d->st>>>(b->sys, b->wsys, b->nwarps, seg_state(A, k),
								 seg_state(A, k + 1), A->lx, A->lu, A->h, b->dt, cK);
			P.pos = seg_state(A, k).pos;
			P.lbase = A->d_lbase + (size_t)k * nsys;
			const int g = grid_for(n, 256);
			switch (A->nt) {
			case 1: ka_pair<1><<<g, 256, 0, d->st>>>(P); break;
			case 2: ka_pair<2><<<g, 256, 0, d->st>>>(P); break;
			case 3: ka_pair<3><<<g, 256, 0, d->st>>>(P); break;
			default: ka_pair<4><<<g, 256, 0, d->st>>>(P); break;
			}
			CKL(d);
		}
	}
	// gradients out
	std::vector<long long> g(2 * ntp * nsys);
	CK(cudaMemcpyAsync(g.data(), A->gslots, sizeof(long long) * 2 * ntp * nsys, cudaMemcpyDeviceToHost,
			   d->st));
	std::vector<double> lx;
	std::vector<int> gid;
	if (dloss_dx0) {
		lx.resize(3 * n);
		gid.resize(n);
		CK(cudaMemcpyAsync(lx.data(), A->lx, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, d->st));
		CK(cudaMemcpyAsync(gid.data(), d->gid, sizeof(int) * n, cudaMemcpyDeviceToHost, d->st));
	}
	CK(cudaStreamSynchronize(d->st));
	long out = 0;
	const int nt = A->nt;
	for (int s = 0; s < nsys; s++) {
		// every ordered type pair gets the gradient of its unordered pair's parameter
		for (int a = 0; a < nt; a++)
			for (int c = 0; c < nt; c++) {
				const int lo = a < c ? a : c, hi = a < c ? c : a;
				const int tu = lo * nt - lo * (lo - 1) / 2 + (hi - lo);
				const size_t o = ((size_t)s * nt + a) * nt + c;
				if (dloss_deps) dloss_deps[o] = (double)g[2 * ntp * s + tu] * FX_ISCALE;
				if (dloss_dsigma) dloss_dsigma[o] = (double)g[2 * ntp * s + ntp + tu] * FX_ISCALE;
			}
		if (dloss_dx0) {
			const BatchSys &S = b->hsys[s];
			for (int t = 0; t < S.n; t++) {
				const int u = gid[S.off + t];
				if (u < 0 || u >= S.n) return batch_fail("sepadj_backward: slot map corrupt", SEPDEV_EINVAL);
				for (int k = 0; k < 3; k++) dloss_dx0[3 * (out + u) + k] = lx[3 * (size_t)(S.off + t) + k];
			}
			out += S.n;
		}
	}
	return SEPDEV_OK;
}

extern "C" int sepadj_backward(sepadj *A, double *dloss_deps, double *dloss_dsigma, double *dloss_dx0)
{
	if (A && A->nt > 1)
		return batch_fail("sepadj_backward: a typed adjoint returns its gradients through "
				  "sepadj_backward_typed", SEPDEV_EINVAL);
	return adj_backward(A, dloss_deps, dloss_dsigma, dloss_dx0);
}

extern "C" int sepadj_backward_typed(sepadj *A, double *dloss_deps, double *dloss_dsigma, double *dloss_dx0)
{
	return adj_backward(A, dloss_deps, dloss_dsigma, dloss_dx0);
}

extern "C" int sepadj_get_state(sepadj *A, int r, double *x, double *v)
{
	if (!A || !A->at_end)
		return batch_fail("sepadj_get_state: call it after sepadj_forward, before sepadj_backward", SEPDEV_EINVAL);
	return sepb_get_state(A->b, r, x, v, NULL);
}
