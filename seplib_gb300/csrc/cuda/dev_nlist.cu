// dev_nlist.cu - cell binning, spatial sort and full Verlet-list build.
//
// Replaces the reference's linked-cell + half-list build
// (source/sepprfrc.c:381-513 and its exclusion variants :517-700) with a
// GB300 pipeline:
//   1. k_bin      cell of every particle straight from the fixed-point high
//                 words (cell = umulhi(x_hi, ncell)), counts with
//                 warp-aggregated atomics (__match_any_sync groups lanes that
//                 share a cell, one atomic per group);
//   2. k_scan     exclusive scan of the counts (one block);
//   3. k_scatter  destination slot = cell start + rank in the cell;
//   4. k_cellsort particles of a cell ordered by user index, so the order and
//                 every floating-point sum after it are run-to-run identical;
//   5. k_gather   all per-particle arrays permuted into cell order;
//   6. k_build    FULL list (both i->j and j->i, so the force pass needs no
//                 atomics), cut-off r^2 < rlist^2 on FP32 minimum-image
//                 separations, exclusions applied, written in warp tiles.
// The cell edge is at least rlist, so the 27-cell stencil covers every pair
// (unlike the reference, whose edge is fixed at setup for skin 0.25).
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "dev_common.cuh"

__global__ void k_bin(long n, const int4 *__restrict__ pos, int ncx, int ncy, int ncz,
		      int *__restrict__ cellof, int *__restrict__ celloff, int *__restrict__ count)
{
	long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
	bool act = s < n;
	int c = -1;
	if (act) {
		int4 p = pos[s];
		int cx = (int)__umulhi((unsigned)p.x, (unsigned)ncx);
		int cy = (int)__umulhi((unsigned)p.y, (unsigned)ncy);
		int cz = (int)__umulhi((unsigned)p.z, (unsigned)ncz);
		c = cx + ncx * (cy + ncy * cz);
	}
	unsigned peers = __match_any_sync(0xffffffffu, c);
	int leader = __ffs(peers) - 1;
	unsigned lane = lane_id();
	int base = 0;
	if (act && (int)lane == leader) base = atomicAdd(&count[c], __popc(peers));
	base = __shfl_sync(0xffffffffu, base, leader);
	if (act) {
		cellof[s] = c;
		celloff[s] = base + __popc(peers & ((1u << lane) - 1u));
	}
}

// exclusive scan of count[0..m) into start[0..m], one block of 1024 threads
__global__ void k_scan(long m, const int *__restrict__ count, int *__restrict__ start)
{
	__shared__ int part[1024];
	const long chunk = (m + blockDim.x - 1) / blockDim.x;
	const long lo = threadIdx.x * chunk, hi = min(m, lo + chunk);
	int s = 0;
	for (long k = lo; k < hi; k++) s += count[k];
	part[threadIdx.x] = s;
	__syncthreads();
	for (int off = 1; off < (int)blockDim.x; off <<= 1) {
		int v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
		__syncthreads();
		part[threadIdx.x] += v;
		__syncthreads();
	}
	int run = threadIdx.x ? part[threadIdx.x - 1] : 0;
	for (long k = lo; k < hi; k++) { start[k] = run; run += count[k]; }
	if (threadIdx.x == blockDim.x - 1) start[m] = part[threadIdx.x];
}

__global__ void k_scatter(long n, const int *__restrict__ cellof, const int *__restrict__ celloff,
			  const int *__restrict__ start, int *__restrict__ perm)
{
	long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
	if (s < n) perm[start[cellof[s]] + celloff[s]] = (int)s;
}

__global__ void k_cellsort(long m, const int *__restrict__ start, const int *__restrict__ gid,
			   int *__restrict__ perm)
{
	long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
	if (c >= m) return;
	int lo = start[c], hi = start[c + 1];
	for (int a = lo + 1; a < hi; a++) {
		int v = perm[a], key = gid[v], b = a - 1;
		while (b >= lo && gid[perm[b]] > key) { perm[b + 1] = perm[b]; b--; }
		perm[b + 1] = v;
	}
}

struct GatherArgs {
	const int *perm;
	const int4 *pos; int4 *pos_o;
	const uint4 *xlo; uint4 *xlo_o;
	const float4 *vhi; float4 *vhi_o;
	const float4 *vlo; float4 *vlo_o;
	const float4 *frc; float4 *frc_o;
	const int4 *cross; int4 *cross_o;
	const int4 *cbase; int4 *cbase_o;
	const int *gid; int *gid_o;
	const float *chg; float *chg_o;
	const int *mol; int *mol_o;
	int4 *xn; int *inv;
	int trigger;
};

__global__ void k_gather(long n, GatherArgs a)
{
	long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
	if (t >= n) return;
	int o = a.perm[t];
	int4 p = a.pos[o];
	a.pos_o[t] = p;
	a.xn[t] = p;
	a.xlo_o[t] = a.xlo[o];
	a.vhi_o[t] = a.vhi[o];
	a.vlo_o[t] = a.vlo[o];
	a.frc_o[t] = a.frc[o];
	int4 c = a.cross[o];
	a.cross_o[t] = c;
	a.cbase_o[t] = a.trigger ? c : a.cbase[o];
	int g = a.gid[o];
	a.gid_o[t] = g;
	a.inv[g] = (int)t;
	a.chg_o[t] = a.chg[o];
	a.mol_o[t] = a.mol[o];
}

__device__ __forceinline__ bool in_csr(const int *__restrict__ st, const int *__restrict__ idx,
				       int who, int what)
{
	for (int k = st[who], e = st[who + 1]; k < e; k++)
		if (idx[k] == what) return true;
	return false;
}

struct BuildArgs {
	const int4 *pos;
	const int *cellstart;
	int nc[3];
	float fs[3];
	float rl2;
	int maxnb;
	int *nl;
	int *ncnt;
	unsigned *flags;
	int excl;
	const int *gid, *mol;
	const int *exs, *exi;   // CSR for the active exclusion mode
};

template <int TPP>
__global__ void __launch_bounds__(128) k_build(long n, BuildArgs a)
{
	long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
	if (i >= n) return;
	constexpr int P = 32 / TPP;
	const int4 pi = a.pos[i];
	const int cx = (int)__umulhi((unsigned)pi.x, (unsigned)a.nc[0]);
	const int cy = (int)__umulhi((unsigned)pi.y, (unsigned)a.nc[1]);
	const int cz = (int)__umulhi((unsigned)pi.z, (unsigned)a.nc[2]);
	int *base = a.nl + (i / P) * (long)a.maxnb * P + (i % P) * TPP;
	const int gi = a.gid[i], mi = a.mol[i];
	int cnt = 0;
	const int lo0 = a.nc[0] >= 3 ? -1 : 0, hi0 = a.nc[0] >= 2 ? 1 : 0;
	const int lo1 = a.nc[1] >= 3 ? -1 : 0, hi1 = a.nc[1] >= 2 ? 1 : 0;
	const int lo2 = a.nc[2] >= 3 ? -1 : 0, hi2 = a.nc[2] >= 2 ? 1 : 0;
	for (int oz = lo2; oz <= hi2; oz++) {
		int zz = cz + oz; zz += (zz < 0) ? a.nc[2] : 0; zz -= (zz >= a.nc[2]) ? a.nc[2] : 0;
		for (int oy = lo1; oy <= hi1; oy++) {
			int yy = cy + oy; yy += (yy < 0) ? a.nc[1] : 0; yy -= (yy >= a.nc[1]) ? a.nc[1] : 0;
			const int row = a.nc[0] * (yy + a.nc[1] * zz);
			for (int ox = lo0; ox <= hi0; ox++) {
				int xx = cx + ox; xx += (xx < 0) ? a.nc[0] : 0; xx -= (xx >= a.nc[0]) ? a.nc[0] : 0;
				const int c = xx + row;
				const int jb = a.cellstart[c], je = a.cellstart[c + 1];
				for (int j = jb; j < je; j++) {
					if (j == (int)i) continue;
					const int4 pj = __ldg(&a.pos[j]);
					const float dx = sep_hi(pi.x, pj.x, a.fs[0]);
					const float dy = sep_hi(pi.y, pj.y, a.fs[1]);
					const float dz = sep_hi(pi.z, pj.z, a.fs[2]);
					const float r2 = dx * dx + dy * dy + dz * dz;
					if (r2 >= a.rl2) continue;
					if (a.excl == SEPDEV_EXCL_SAMEMOL) {
						if (mi != -1 && mi == a.mol[j]) continue;
					} else if (a.excl != SEPDEV_EXCL_NONE) {
						const int gj = a.gid[j];
						if (in_csr(a.exs, a.exi, gi, gj) || in_csr(a.exs, a.exi, gj, gi)) continue;
					}
					if (cnt < a.maxnb) base[(cnt / TPP) * 32 + (cnt % TPP)] = j;
					cnt++;
				}
			}
		}
	}
	a.ncnt[i] = cnt < a.maxnb ? cnt : a.maxnb;
	if (cnt > a.maxnb) atomicOr(&a.flags[0], 1u);
	atomicMax(&a.flags[1], (unsigned)cnt);
}

static int grow(sepdev *d, void **p, size_t bytes, size_t *cap)
{
	if (*p && *cap >= bytes) return SEPDEV_OK;
	if (*p) cudaFree(*p);
	*p = NULL;
	cudaError_t e = cudaMalloc(p, bytes);
	if (e != cudaSuccess) { sepdev_set_error("cudaMalloc(list)", e); *cap = 0; return SEPDEV_ENOMEM; }
	*cap = bytes;
	(void)d;
	return SEPDEV_OK;
}

static int launch_build(sepdev *d, const BuildArgs &a)
{
	const int B = 128;
	switch (d->tpp) {
	case 1: k_build<1><<<grid_for(d->n, B), B, 0, d->st>>>(d->n, a); break;
	case 2: k_build<2><<<grid_for(d->n, B), B, 0, d->st>>>(d->n, a); break;
	case 4: k_build<4><<<grid_for(d->n, B), B, 0, d->st>>>(d->n, a); break;
	default: k_build<8><<<grid_for(d->n, B), B, 0, d->st>>>(d->n, a); break;
	}
	CKL(d);
	return SEPDEV_OK;
}

// Copy the gathered arrays back into the primary buffers, so buffer
// addresses never change (graph-captured launches keep valid arguments).
struct CopyArgs {
	const int4 *pos_s; int4 *pos_d;
	const uint4 *xlo_s; uint4 *xlo_d;
	const float4 *vhi_s; float4 *vhi_d;
	const float4 *vlo_s; float4 *vlo_d;
	const float4 *frc_s; float4 *frc_d;
	const int4 *cross_s; int4 *cross_d;
	const int4 *cbase_s; int4 *cbase_d;
	const int *gid_s; int *gid_d;
	const float *chg_s; float *chg_d;
	const int *mol_s; int *mol_d;
};

__global__ void k_copyback(long n, CopyArgs a)
{
	long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
	if (t >= n) return;
	a.pos_d[t] = a.pos_s[t];
	a.xlo_d[t] = a.xlo_s[t];
	a.vhi_d[t] = a.vhi_s[t];
	a.vlo_d[t] = a.vlo_s[t];
	a.frc_d[t] = a.frc_s[t];
	a.cross_d[t] = a.cross_s[t];
	a.cbase_d[t] = a.cbase_s[t];
	a.gid_d[t] = a.gid_s[t];
	a.chg_d[t] = a.chg_s[t];
	a.mol_d[t] = a.mol_s[t];
}

// Cell grid for cut-off rlist: edge >= rlist, total cells bounded by 2n + 64.
static int cell_grid(sepdev *d, double rlist)
{
	for (int k = 0; k < 3; k++) {
		int c = (int)floor(d->L[k] / rlist);
		d->ncell[k] = c < 1 ? 1 : c;
	}
	while ((long)d->ncell[0] * d->ncell[1] * d->ncell[2] > 2 * d->n + 64) {
		int k = 0;
		for (int q = 1; q < 3; q++) if (d->ncell[q] > d->ncell[k]) k = q;
		d->ncell[k] = d->ncell[k] > 1 ? d->ncell[k] - 1 : 1;
	}
	d->ncells = (long)d->ncell[0] * d->ncell[1] * d->ncell[2];
	if (d->ncells + 1 > d->cap_cells) {
		if (d->cellcount) cudaFree(d->cellcount);
		if (d->cellstart) cudaFree(d->cellstart);
		d->cellcount = d->cellstart = NULL;
		CK(cudaMalloc((void **)&d->cellcount, sizeof(int) * (d->ncells + 1)));
		CK(cudaMalloc((void **)&d->cellstart, sizeof(int) * (d->ncells + 1)));
		d->cap_cells = d->ncells + 1;
	}
	return SEPDEV_OK;
}

// Cell binning and permutation into cell order (steps 1-5), reading and
// leaving the positions in buffer `parity`.  Asynchronous; capturable.
int sepdev_sort_async(sepdev *d, int parity, int trigger)
{
	const long n = d->n;
	const int B = 256;
	CK(cudaMemsetAsync(d->cellcount, 0, sizeof(int) * d->ncells, d->st));
	k_bin<<<grid_for(n, B), B, 0, d->st>>>(n, d->pos[parity], d->ncell[0], d->ncell[1],
					     d->ncell[2], d->cellof, d->celloff, d->cellcount);
	CKL(d);
	k_scan<<<1, 1024, 0, d->st>>>(d->ncells, d->cellcount, d->cellstart);
	CKL(d);
	k_scatter<<<grid_for(n, B), B, 0, d->st>>>(n, d->cellof, d->celloff, d->cellstart, d->perm);
	CKL(d);
	k_cellsort<<<grid_for(d->ncells, B), B, 0, d->st>>>(d->ncells, d->cellstart, d->gid, d->perm);
	CKL(d);
	GatherArgs g;
	const int o = parity ^ 1;
	g.perm = d->perm;
	g.pos = d->pos[parity]; g.pos_o = d->pos[o];
	g.xlo = d->xlo; g.xlo_o = d->xlo_b;
	g.vhi = d->vhi; g.vhi_o = d->vhi_b;
	g.vlo = d->vlo; g.vlo_o = d->vlo_b;
	g.frc = d->frc; g.frc_o = d->frc_b;
	g.cross = d->cross; g.cross_o = d->cross_b;
	g.cbase = d->cbase; g.cbase_o = d->cbase_b;
	g.gid = d->gid; g.gid_o = d->gid_b;
	g.chg = d->charge; g.chg_o = d->charge_b;
	g.mol = d->mol; g.mol_o = d->mol_b;
	g.xn = d->xn; g.inv = d->inv;
	g.trigger = trigger;
	k_gather<<<grid_for(n, B), B, 0, d->st>>>(n, g);
	CKL(d);
	CopyArgs c;
	c.pos_s = d->pos[o]; c.pos_d = d->pos[parity];
	c.xlo_s = d->xlo_b; c.xlo_d = d->xlo;
	c.vhi_s = d->vhi_b; c.vhi_d = d->vhi;
	c.vlo_s = d->vlo_b; c.vlo_d = d->vlo;
	c.frc_s = d->frc_b; c.frc_d = d->frc;
	c.cross_s = d->cross_b; c.cross_d = d->cross;
	c.cbase_s = d->cbase_b; c.cbase_d = d->cbase;
	c.gid_s = d->gid_b; c.gid_d = d->gid;
	c.chg_s = d->charge_b; c.chg_d = d->charge;
	c.mol_s = d->mol_b; c.mol_d = d->mol;
	k_copyback<<<grid_for(n, B), B, 0, d->st>>>(n, c);
	CKL(d);
	return SEPDEV_OK;
}

static int list_capacity(sepdev *d, int maxnb)
{
	const int P = 32 / d->tpp;
	maxnb = ((maxnb + 7) / 8) * 8;
	const size_t tiles = (size_t)((d->n + P - 1) / P);
	const size_t bytes = tiles * (size_t)P * (size_t)maxnb * sizeof(int);
	int rc = grow(d, (void **)&d->nl, bytes, &d->cap_nl);
	if (rc) return rc;
	d->maxnb = maxnb;
	return SEPDEV_OK;
}

int sepdev_build_args(sepdev *d, BuildArgs *a, int parity)
{
	a->pos = d->pos[parity];
	a->cellstart = d->cellstart;
	for (int k = 0; k < 3; k++) { a->nc[k] = d->ncell[k]; a->fs[k] = d->fscale[k]; }
	a->rl2 = (float)(d->rlist * d->rlist);
	a->maxnb = d->maxnb;
	a->nl = d->nl;
	a->ncnt = d->ncnt;
	a->flags = d->flags;
	a->excl = d->excl;
	a->gid = d->gid;
	a->mol = d->mol;
	a->exs = d->excl == SEPDEV_EXCL_BONDS ? d->exb_start : d->exa_start;
	a->exi = d->excl == SEPDEV_EXCL_BONDS ? d->exb_idx : d->exa_idx;
	return SEPDEV_OK;
}

// List build from the sorted positions of buffer `parity`; clears the
// overflow flag first.  Asynchronous; capturable.
int sepdev_build_async(sepdev *d, int parity)
{
	CK(cudaMemsetAsync(d->flags, 0, sizeof(unsigned) * 2, d->st));
	BuildArgs a;
	sepdev_build_args(d, &a, parity);
	return launch_build(d, a);
}

// Host-driven rebuild: sort, build, check the capacity and grow it when a
// particle overflowed (synchronous).
extern "C" int sepdev_build_list(sepdev *d, double rlist, int excl, int trigger)
{
	if (!(rlist > 0)) return SEPDEV_EINVAL;
	if ((excl == SEPDEV_EXCL_BONDS || excl == SEPDEV_EXCL_ALLBONDED) && !d->has_excl)
		excl = SEPDEV_EXCL_NONE;
	d->rlist = rlist;
	d->excl = excl;
	int rc;
	if ((rc = cell_grid(d, rlist))) return rc;
	if ((rc = sepdev_sort_async(d, d->cur, trigger))) return rc;
	if (d->maxnb == 0) {
		const double vol = d->L[0] * d->L[1] * d->L[2];
		const double est = 4.18879020479 * rlist * rlist * rlist * (double)d->n / vol;
		if ((rc = list_capacity(d, (int)(1.35 * est) + 32))) return rc;
	}
	for (int attempt = 0; attempt < 4; attempt++) {
		if ((rc = sepdev_build_async(d, d->cur))) return rc;
		unsigned fl[2];
		CK(cudaMemcpyAsync(fl, d->flags, sizeof fl, cudaMemcpyDeviceToHost, d->st));
		CK(cudaStreamSynchronize(d->st));
		if (!(fl[0] & 1u)) { d->list_valid = 1; return SEPDEV_OK; }
		if ((rc = list_capacity(d, (int)(fl[1] * 1.25) + 16))) return rc;
	}
	return SEPDEV_EOVERFLOW;
}

// Grow the list for a count the device reported (used after an in-graph overflow).
int sepdev_grow_list(sepdev *d, int needed)
{
	return list_capacity(d, (int)(needed * 1.25) + 16);
}

extern "C" int sepdev_list_stats(sepdev *d, int *maxcount, double *meancount, int *capacity)
{
	int *h = (int *)malloc(sizeof(int) * d->n);
	if (!h) return SEPDEV_ENOMEM;
	CK(cudaMemcpyAsync(h, d->ncnt, sizeof(int) * d->n, cudaMemcpyDeviceToHost, d->st));
	CK(cudaStreamSynchronize(d->st));
	long s = 0; int mx = 0;
	for (long i = 0; i < d->n; i++) { s += h[i]; if (h[i] > mx) mx = h[i]; }
	free(h);
	if (maxcount) *maxcount = mx;
	if (meancount) *meancount = (double)s / d->n;
	if (capacity) *capacity = d->maxnb;
	return SEPDEV_OK;
}

static int cmp_pair(const void *a, const void *b)
{
	const int *x = (const int *)a, *y = (const int *)b;
	if (x[0] != y[0]) return x[0] < y[0] ? -1 : 1;
	if (x[1] != y[1]) return x[1] < y[1] ? -1 : 1;
	return 0;
}

extern "C" long sepdev_list_pairs(sepdev *d, int *pairs, long cap)
{
	if (!d->list_valid) return -1;
	const long n = d->n;
	const int P = 32 / d->tpp;
	const size_t tiles = (size_t)((n + P - 1) / P);
	const size_t len = tiles * P * (size_t)d->maxnb;
	int *nl = (int *)malloc(sizeof(int) * len), *cnt = (int *)malloc(sizeof(int) * n);
	int *gid = (int *)malloc(sizeof(int) * n);
	if (!nl || !cnt || !gid) { free(nl); free(cnt); free(gid); return -2; }
	cudaMemcpyAsync(nl, d->nl, sizeof(int) * len, cudaMemcpyDeviceToHost, d->st);
	cudaMemcpyAsync(cnt, d->ncnt, sizeof(int) * n, cudaMemcpyDeviceToHost, d->st);
	cudaMemcpyAsync(gid, d->gid, sizeof(int) * n, cudaMemcpyDeviceToHost, d->st);
	if (cudaStreamSynchronize(d->st) != cudaSuccess) { free(nl); free(cnt); free(gid); return -3; }
	long np = 0;
	for (long i = 0; i < n; i++) {
		const int *base = nl + (i / P) * (size_t)d->maxnb * P + (i % P) * d->tpp;
		for (int k = 0; k < cnt[i]; k++) {
			int j = base[(k / d->tpp) * 32 + (k % d->tpp)];
			int gi = gid[i], gj = gid[j];
			if (gi < gj) {
				if (np < cap) { pairs[2 * np] = gi; pairs[2 * np + 1] = gj; }
				np++;
			}
		}
	}
	if (np <= cap) qsort(pairs, np, 2 * sizeof(int), cmp_pair);
	free(nl); free(cnt); free(gid);
	return np;
}

extern "C" int sepdev_set_tpp(sepdev *d, int tpp)
{
	if (tpp != 1 && tpp != 2 && tpp != 4) return SEPDEV_EINVAL;
	d->tpp = tpp;
	d->list_valid = 0;
	return SEPDEV_OK;
}

extern "C" int sepdev_get_tpp(sepdev *d) { return d->tpp; }
