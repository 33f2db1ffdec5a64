// dev_batch.cu - many independent LJ systems stepped together (sepb_* API).
//
// Each system is the prgs loop of the reference (pair forces, Nose-Hoover,
// leap-frog; source/sepprfrc.c:743-1000, source/sepintgr.c:42-88,149-168)
// with its own box, density, temperature, thermostat and neighbour-list
// updates.  A per-system launch would leave the GPU idle (a 108-particle
// system is one block), so the systems share one set of device arrays and
// every step is one batched fused kernel plus one decision kernel with a warp
// per system, in one CUDA graph:
//
//   WHILE (iterations left) {
//     IF (some system asked for a rebuild) { sort + list build of those systems }
//     batched fused step (forces, friction, leap-frog, per-system sums)
//     decision (per system: thermostat, skin test, rebuild flag; sets the IF)
//     ... RUN_UNROLL_B steps
//   }
//
// A system is rebuilt exactly when its own skin test fires, as a
// single-system run would be, and every per-particle operation is the one
// of the single-system kernels, so each system of a batch reproduces the
// single-system path.
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <vector>
#include "dev_common.cuh"
#include "dev_batch.cuh"
#include "dev_cellsort.cuh"
#include "sepbatch.h"
#include "sepdef.h"

#define RUN_UNROLL_B 8

int sepdev_grow_list_to(sepdev *d, int maxnb);

// ---- the rebuild of flagged systems ----------------------------------------

// one block per system: a flagged system appends its 32-slot warps to the
// list of warps the batched list build steps through (a fixed grid, so the
// build of a few systems runs as a few well-filled waves instead of a warp
// per slot group of every system, most leaving at once).  A warp's list
// depends on nothing but the warp, so the order of the list changes no
// result.
__global__ void kb_compact(const BatchSys *sys, const unsigned *flag, int *fw, int *cnt)
{
	const int s = blockIdx.x;
	if (!flag[s]) return;                          // uniform over the block
	const BatchSys S = sys[s];
	const int nw = S.npad / 32;
	__shared__ int base;
	if (threadIdx.x == 0) base = atomicAdd(cnt, nw);
	__syncthreads();
	for (int k = threadIdx.x; k < nw; k += blockDim.x) fw[base + k] = S.off / 32 + k;
}

__global__ void kb_bin(const BatchSys *sys, const int *wsys, int nwarps, const unsigned *flag,
		       const int4 *pos, int *cellof, int *celloff, int *count)
{
	const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
	const long wg = t >> 5;
	if (wg >= nwarps) return;
	const int s = wsys[wg];
	if (!flag[s]) return;                          // uniform over the warp
	const BatchSys S = sys[s];
	int c;
	if (t - S.off < S.n) {
		const int4 p = pos[t];
		const int cx = (int)__umulhi((unsigned)p.x, (unsigned)S.nc[0]);
		const int cy = (int)__umulhi((unsigned)p.y, (unsigned)S.nc[1]);
		const int cz = (int)__umulhi((unsigned)p.z, (unsigned)S.nc[2]);
		c = S.coff + cx + S.nc[0] * (cy + S.nc[1] * cz);
	} else {
		c = S.coff + S.ncell;                   // the padding cell
	}
	const unsigned peers = __match_any_sync(0xffffffffu, c);
	const int leader = __ffs(peers) - 1;
	const int lane = threadIdx.x & 31;
	int base = 0;
	if (lane == leader) base = atomicAdd(&count[c], __popc(peers));
	base = __shfl_sync(0xffffffffu, base, leader);
	cellof[t] = c;
	celloff[t] = base + __popc(peers & ((1u << lane) - 1u));
}

// one block per system: exclusive scan of its ncell + 1 counts into slot
// starts (the system's slots begin at off)
__global__ void kb_scan(const BatchSys *sys, const unsigned *flag, const int *count, int *start)
{
	const int s = blockIdx.x;
	if (!flag[s]) return;
	const BatchSys S = sys[s];
	__shared__ int carry;
	__shared__ int wsum[32];
	const int t = threadIdx.x, lane = t & 31, w = t >> 5;
	if (t == 0) carry = S.off;
	const int m = S.ncell + 1;
	for (int base = 0; base < m; base += blockDim.x) {
		const int k = base + t;
		const int v = k < m ? count[S.coff + k] : 0;
		int x = v;
		for (int o = 1; o < 32; o <<= 1) {
			const int y = __shfl_up_sync(0xffffffffu, x, o);
			if (lane >= o) x += y;
		}
		__syncthreads();
		if (lane == 31) wsum[w] = x;
		__syncthreads();
		if (w == 0) {
			int ws = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0;
			for (int o = 1; o < 32; o <<= 1) {
				const int y = __shfl_up_sync(0xffffffffu, ws, o);
				if (lane >= o) ws += y;
			}
			wsum[lane] = ws;
		}
		__syncthreads();
		const int c0 = carry;
		if (k < m) start[S.coff + k] = c0 + (w ? wsum[w - 1] : 0) + x - v;
		__syncthreads();
		if (t == 0) carry = c0 + wsum[(blockDim.x >> 5) - 1];
	}
	__syncthreads();
	if (t == 0) start[S.coff + m] = carry;
}

__global__ void kb_scatter(const int *wsys, int nwarps, const unsigned *flag, const int *cellof,
			   const int *celloff, const int *start, int *perm)
{
	const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
	const long wg = t >> 5;
	if (wg >= nwarps || !flag[wsys[wg]]) return;
	perm[start[cellof[t]] + celloff[t]] = (int)t;
}

// a warp per cell: members ordered by x, ties by their index in the
// system (dev_cellsort.cuh); launched with 256 threads
__global__ void __launch_bounds__(256) kb_cellsort(long ncells, const int *csys, const unsigned *flag,
						   const int *start, const int *gid, const int4 *pos, int *perm)
{
	__shared__ unsigned long long sk[8][CS_MAX];
	__shared__ int sv[8][CS_MAX];
	const long c = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
	if (c >= ncells) return;
	const int s = csys[c];
	if (s < 0 || !flag[s]) return;
	const int w = threadIdx.x >> 5;
	const int lo = start[c];
	cell_sort_warp(lo, start[c + 1] - lo, gid, pos, perm, sk[w], sv[w]);
}

struct BGather {
	const BatchSys *sys;
	const int *wsys;
	const unsigned *flag;
	int nwarps;
	const int *perm;
	const int4 *pos; int4 *pos_o;
	const uint4 *xlo; uint4 *xlo_o;
	const float4 *vhi; float4 *vhi_o;
	const float4 *vlo; float4 *vlo_o;
	const float4 *frc; float4 *frc_o;
	const int4 *cross; int4 *cross_o;
	const int4 *cbase; int4 *cbase_o;
	const int *gid; int *gid_o;
	int4 *xn; int *inv;
};

__global__ void kb_gather(BGather a)
{
	const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
	const long wg = t >> 5;
	if (wg >= a.nwarps) return;
	const int s = a.wsys[wg];
	if (!a.flag[s]) return;
	const int o = a.perm[t];
	const int4 p = a.pos[o];
	a.pos_o[t] = p;
	a.xn[t] = p;
	a.xlo_o[t] = a.xlo[o];
	a.vhi_o[t] = a.vhi[o];
	a.vlo_o[t] = a.vlo[o];
	a.frc_o[t] = a.frc[o];
	const int4 c = a.cross[o];
	a.cross_o[t] = c;
	a.cbase_o[t] = c;                          // every batched rebuild is a skin-triggered one
	const int g = a.gid[o];
	a.gid_o[t] = g;
	const BatchSys S = a.sys[s];
	if (g < S.n) a.inv[S.off + g] = (int)t;
}

__global__ void kb_copyback(BGather a)
{
	const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
	const long wg = t >> 5;
	if (wg >= a.nwarps || !a.flag[a.wsys[wg]]) return;
	int4 *pos_d = (int4 *)a.pos;
	uint4 *xlo_d = (uint4 *)a.xlo;
	float4 *vhi_d = (float4 *)a.vhi, *vlo_d = (float4 *)a.vlo, *frc_d = (float4 *)a.frc;
	int4 *cross_d = (int4 *)a.cross, *cbase_d = (int4 *)a.cbase;
	int *gid_d = (int *)a.gid;
	pos_d[t] = a.pos_o[t];
	xlo_d[t] = a.xlo_o[t];
	vhi_d[t] = a.vhi_o[t];
	vlo_d[t] = a.vlo_o[t];
	frc_d[t] = a.frc_o[t];
	cross_d[t] = a.cross_o[t];
	cbase_d[t] = a.cbase_o[t];
	gid_d[t] = a.gid_o[t];
}

// ---- the per-system decision ------------------------------------------------

// a warp per system (decide_warp of the single-system loop), then the last
// system to finish sets the graph's handles for all of them
__global__ void kb_decide(BatchDecide a)
{
	const unsigned FULL = 0xffffffffu;
	const int s = (int)((blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5);
	const int lane = threadIdx.x & 31;
	if (s >= a.nsys) return;
	BatchRun *run = a.run;
	const bool abort = run->abort || (__ldcg(a.oflow) & 1u);
	if (!abort) {
		BatchState *st = &a.bs[s];
		long long *slot = a.slots + (long)s * SLOT_FIELDS;
		const long long v = __ldcg(slot + lane);
		const double val = (lane == SLOT_MAXD2) ? (double)__uint_as_float((unsigned)v) : (double)v * FX_ISCALE;
		st->last[lane] = val;
		slot[lane] = 0;
		const double sumv2 = __shfl_sync(FULL, val, SLOT_SUMV2);
		const double maxd2 = __shfl_sync(FULL, val, SLOT_MAXD2);
		// loss term of this step: epot + p, p = tr(kin_P + pot_P) / 3V
		const double ep = __shfl_sync(FULL, val, SLOT_EPOT0);
		double tr = 0.0;
		for (int k = 0; k < 3; k++) {
			const int dk = k == 0 ? 0 : (k == 1 ? 3 : 5);
			tr += __shfl_sync(FULL, val, SLOT_KINP + dk) + __shfl_sync(FULL, val, SLOT_POTP + dk);
		}
		if (lane == 0) {
			if (a.loss_scale != 0.0) {
				const double V = a.sys[s].L * a.sys[s].L * a.sys[s].L;
				st->loss += a.loss_scale * (ep + tr / (3.0 * V));
			}
			st->sumv2 = sumv2;
			st->alpha_last = st->alpha;
			if (a.nh) {
				const double ekin = __ddiv_rn(__dmul_rn(0.5, sumv2), (double)a.sys[s].n);
				const double temp = __dmul_rn(0.666667, ekin);
				st->alpha = __dadd_rn(st->alpha,
						      __dmul_rn(a.dt_tau2, __dsub_rn(__ddiv_rn(temp, a.sys[s].T0), 1.0)));
			}
			const int trig = ((float)maxd2 > a.thr2) || st->force_trig;
			st->force_trig = 0;
			st->last_trig = trig;
			st->ntrig += trig;
			a.flag[s] = trig;
			if (trig) atomicOr(&run->any, 1u);
		}
	}
	if (lane != 0) return;
	__threadfence();
	if (atomicAdd(&run->arrive, 1u) != (unsigned)a.nsys - 1) return;
	__threadfence();
	run->arrive = 0;
	if (abort) {
		run->abort = 1;
		if (a.use_handles) {
			cudaGraphSetConditional(a.h_next, 0);
			if (a.pair_end) cudaGraphSetConditional(a.h_while, 0);
		}
		return;
	}
	const unsigned any = atomicExch(&run->any, 0u);
	run->last_any = any;
	run->done += 1;
	if (a.use_handles) {
		cudaGraphSetConditional(a.h_next, any);
		if (a.pair_end) {
			run->remaining -= 1;
			cudaGraphSetConditional(a.h_while, run->remaining > 0 ? 1u : 0u);
		}
	}
}

__global__ void kb_flush(uint4 *buf, long n16, unsigned tag)
{
	for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n16; i += (long)gridDim.x * blockDim.x)
		buf[i] = make_uint4((unsigned)i, tag, (unsigned)i ^ tag, 0u);
}

// ---- host side ---------------------------------------------------------------


void batch_to_fixed(double x, double L, unsigned *hi, unsigned *lo)
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

double batch_from_fixed(unsigned hi, unsigned lo, double L)
{
	return (ldexp((double)hi, -32) + ldexp((double)lo, -64)) * L;
}

int batch_fail(const char *what, int rc)
{
	sepdev_set_error(what, cudaErrorInvalidValue);
	return rc;
}

extern "C" void sepb_destroy(sepb *b)
{
	if (!b) return;
	if (b->d) cudaStreamSynchronize(b->d->st);
	if (b->exec) cudaGraphExecDestroy(b->exec);
	if (b->graph) cudaGraphDestroy(b->graph);
	void *dv[] = {b->sys, b->wsys, b->csys, b->flag, b->cellcount, b->cellstart, b->slots, b->bs, b->run,
		      b->flush_buf, b->wstep, b->fw, b->fcnt};
	for (size_t k = 0; k < sizeof dv / sizeof dv[0]; k++)
		if (dv[k]) cudaFree(dv[k]);
	if (b->h_bs) cudaFreeHost(b->h_bs);
	if (b->h_run) cudaFreeHost(b->h_run);
	if (b->d) sepdev_destroy(b->d);
	delete b;
}

#define BCK(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) { sepdev_set_error(#call, e_); \
	sepb_destroy(b); return NULL; } } while (0)

// typed: the per-type-pair kernel, which takes one lane per particle
static sepb *batch_make(int nsys, const int *npart, const double *L, double rc, double skin, double dt,
			const double *ljparam, int typed)
{
	if (nsys <= 0 || !npart || !L || !(rc > 0) || !(skin >= 0) || !(dt > 0)) {
		batch_fail("sepb_create: invalid arguments", SEPDEV_EINVAL);
		return NULL;
	}
	sepb *b = new sepb();          // value-initialised: pointers and counters start at zero
	b->nsys = nsys;
	b->rc = rc; b->skin = skin; b->dt = dt;
	b->tau = 10.0;
	if (ljparam) {
		if (ljparam[0] > rc) { batch_fail("sepb_create: LJ cut-off larger than rc", SEPDEV_EINVAL); delete b; return NULL; }
		b->cf = ljparam[0]; b->eps = ljparam[1]; b->sigma = ljparam[2]; b->aw = ljparam[3];
		b->ushift = -4.0 * b->eps * (pow(b->sigma / b->cf, 12.) - b->aw * pow(b->sigma / b->cf, 6.));
	} else {
		// sep_lj_shift: unit LJ, shifted to zero at 2.5 (source/sepmisc.c:115-135)
		b->cf = rc; b->eps = 1.0; b->sigma = 1.0; b->aw = 1.0; b->ushift = SEP_LJCF2;
	}
	const double rlist = rc + skin;
	b->hsys.resize(nsys);
	b->have.assign(nsys, 0);
	b->fresh.assign(nsys, 0);
	b->nupd.assign(nsys, 0u);
	b->alpha0.assign(nsys, 0.0);
	long off = 0, coff = 0;
	std::vector<int> hw, hc;
	std::vector<int4> hstep;
	for (int s = 0; s < nsys; s++) {
		BatchSys &S = b->hsys[s];
		if (npart[s] <= 0 || !(L[s] > 0)) { batch_fail("sepb_create: empty system or box", SEPDEV_EINVAL); delete b; return NULL; }
		S.n = npart[s];
		S.npad = (S.n + 31) & ~31;
		S.off = (int)off;
		S.L = L[s];
		S.fs = (float)(L[s] / 4294967296.0);
		// from the FP32 sigma^2 and cut-off the single-system path holds, so a
		// system computes with the same constants in a batch and alone
		S.sc = lj_scale(L[s], (double)(float)(b->sigma * b->sigma), (double)(float)(b->cf * b->cf));
		const double sc = dt * 18446744073709551616.0 / L[s];
		S.shi = (float)sc;
		S.slo = (float)(sc - (double)S.shi);
		// the kernel parameters of the system's size class
		sepdev_tuning_for(S.n, &S.team, &S.groups, &S.cellf);
		if (typed) S.team = 1;
		int nc = (int)floor(L[s] / (rlist * S.cellf));
		if (nc < 1) nc = 1;
		// the single-system grid bound: at most 2n + 64 cells
		int ncs[3] = {nc, nc, nc};
		while ((long)ncs[0] * ncs[1] * ncs[2] > 2L * S.n + 64) {
			int k = 0;
			for (int q = 1; q < 3; q++) if (ncs[q] > ncs[k]) k = q;
			ncs[k] = ncs[k] > 1 ? ncs[k] - 1 : 1;
		}
		for (int k = 0; k < 3; k++) S.nc[k] = ncs[k];
		S.ncell = ncs[0] * ncs[1] * ncs[2];
		S.coff = (int)coff;
		S.T0 = 1.0;
		for (int w = 0; w < S.npad / 32; w++) hw.push_back(s);
		for (int k = 0; k < S.npad; k += 32 / S.team)
			hstep.push_back(make_int4(s, (int)off + k, S.team, S.groups));
		for (int c = 0; c < S.ncell + 1; c++) hc.push_back(s);
		hc.push_back(-1);                       // the end entry
		off += S.npad;
		coff += S.ncell + 2;
		if (off > (1L << 30)) { batch_fail("sepb_create: too many particles", SEPDEV_EINVAL); delete b; return NULL; }
	}
	b->ntot = off;
	b->nwarps = (int)(off / 32);
	b->ncells = coff;
	int rc0 = sepdev_create(&b->d, b->ntot);
	if (rc0) { sepb_destroy(b); return NULL; }
	sepdev *d = b->d;
	for (int k = 0; k < 3; k++) { d->L[k] = 1.0; d->fscale[k] = (float)(1.0 / 4294967296.0); }
	BCK(cudaMalloc((void **)&b->sys, sizeof(BatchSys) * nsys));
	BCK(cudaMalloc((void **)&b->wsys, sizeof(int) * b->nwarps));
	b->nstepw = (int)hstep.size();
	BCK(cudaMalloc((void **)&b->wstep, sizeof(int4) * b->nstepw));
	BCK(cudaMemcpy(b->wstep, hstep.data(), sizeof(int4) * b->nstepw, cudaMemcpyHostToDevice));
	BCK(cudaMalloc((void **)&b->csys, sizeof(int) * b->ncells));
	BCK(cudaMalloc((void **)&b->flag, sizeof(unsigned) * nsys));
	BCK(cudaMalloc((void **)&b->fw, sizeof(int) * b->nwarps));
	BCK(cudaMalloc((void **)&b->fcnt, sizeof(int)));
	BCK(cudaMalloc((void **)&b->cellcount, sizeof(int) * b->ncells));
	BCK(cudaMalloc((void **)&b->cellstart, sizeof(int) * b->ncells));
	BCK(cudaMalloc((void **)&b->slots, sizeof(long long) * SLOT_FIELDS * nsys));
	BCK(cudaMalloc((void **)&b->bs, sizeof(BatchState) * nsys));
	BCK(cudaMalloc((void **)&b->run, sizeof(BatchRun)));
	BCK(cudaMallocHost((void **)&b->h_bs, sizeof(BatchState) * nsys));
	BCK(cudaMallocHost((void **)&b->h_run, sizeof(BatchRun)));
	BCK(cudaMemcpy(b->sys, b->hsys.data(), sizeof(BatchSys) * nsys, cudaMemcpyHostToDevice));
	BCK(cudaMemcpy(b->wsys, hw.data(), sizeof(int) * b->nwarps, cudaMemcpyHostToDevice));
	BCK(cudaMemcpy(b->csys, hc.data(), sizeof(int) * b->ncells, cudaMemcpyHostToDevice));
	BCK(cudaMemset(b->slots, 0, sizeof(long long) * SLOT_FIELDS * nsys));
	BCK(cudaMemset(b->flag, 0, sizeof(unsigned) * nsys));
	memset(b->h_bs, 0, sizeof(BatchState) * nsys);
	memset(b->h_run, 0, sizeof(BatchRun));
	// list capacity from the densest system: 1.6 x the mean full-list length + 32
	double rho_max = 0.0;
	for (int s = 0; s < nsys; s++) {
		const double rho = b->hsys[s].n / (L[s] * L[s] * L[s]);
		if (rho > rho_max) rho_max = rho;
	}
	const double nbar = 4.0 / 3.0 * M_PI * rlist * rlist * rlist * rho_max;
	int maxnb = (int)(1.6 * nbar) + 32;
	if (maxnb > 1024) maxnb = 1024;
	if (sepdev_grow_list_to(d, maxnb)) { sepb_destroy(b); return NULL; }
	return b;
}

extern "C" sepb *sepb_create(int nsys, const int *npart, const double *L, double rc, double skin,
			     double dt, const double *ljparam)
{
	return batch_make(nsys, npart, L, rc, skin, dt, ljparam, 0);
}

extern "C" int sepb_set_state(sepb *b, int s, const double *x, const double *v, const double *m)
{
	if (!b || s < 0 || s >= b->nsys || !x || !v) return batch_fail("sepb_set_state: invalid arguments", SEPDEV_EINVAL);
	const BatchSys &S = b->hsys[s];
	sepdev *d = b->d;
	const int n = S.n, np = S.npad;
	std::vector<int4> hp(np), hc(np, make_int4(0, 0, 0, 0));
	std::vector<uint4> hl(np);
	std::vector<float4> hvh(np), hvl(np), hf(np, make_float4(0.f, 0.f, 0.f, 0.f));
	std::vector<int> hg(np), hz(np, -1);
	std::vector<float> hq(np, 0.f);
	double sv2 = 0.0;
	for (int i = 0; i < np; i++) {
		if (i < n) {
			unsigned h[3], l[3];
			for (int k = 0; k < 3; k++) batch_to_fixed(x[3 * i + k], S.L, &h[k], &l[k]);
			hp[i] = make_int4((int)h[0], (int)h[1], (int)h[2], 0);
			hl[i] = make_uint4(l[0], l[1], l[2], 0u);
			float vh[3], vl[3];
			const double mi = m ? m[i] : 1.0;
			for (int k = 0; k < 3; k++) {
				vh[k] = (float)v[3 * i + k];
				vl[k] = (float)(v[3 * i + k] - (double)vh[k]);
				sv2 += v[3 * i + k] * v[3 * i + k] * mi;
			}
			hvh[i] = make_float4(vh[0], vh[1], vh[2], (float)mi);
			hvl[i] = make_float4(vl[0], vl[1], vl[2], (float)(1.0 / mi));
		} else {
			// inert padding: never binned into a real cell, never integrated
			hp[i] = make_int4(0, 0, 0, 0);
			hl[i] = make_uint4(0u, 0u, 0u, 0u);
			hvh[i] = make_float4(0.f, 0.f, 0.f, 1.f);
			hvl[i] = make_float4(0.f, 0.f, 0.f, 1.f);
		}
		hg[i] = i;
	}
	const size_t o = (size_t)S.off;
#define UPB(dst, src) do { cudaError_t e_ = cudaMemcpy(dst + o, src.data(), sizeof(src[0]) * np, cudaMemcpyHostToDevice); \
	if (e_ != cudaSuccess) { sepdev_set_error("sepb_set_state", e_); return SEPDEV_ECUDA; } } while (0)
	UPB(d->pos[0], hp); UPB(d->pos[1], hp); UPB(d->xn, hp); UPB(d->xlo, hl);
	UPB(d->vhi, hvh); UPB(d->vlo, hvl); UPB(d->frc, hf);
	UPB(d->cross, hc); UPB(d->cbase, hc); UPB(d->gid, hg); UPB(d->inv, hg);
	UPB(d->mol, hz); UPB(d->charge, hq);
#undef UPB
	BatchState &st = b->h_bs[s];
	memset(&st, 0, sizeof st);
	st.sumv2 = sv2;
	st.alpha_last = b->alpha0[s];
	// a fresh system reports a list update after its first step, as a
	// seplib program does (sep_init leaves xn unset)
	st.force_trig = 1;
	b->nupd[s] = 0;
	b->have[s] = 1;
	b->fresh[s] = 1;
	b->list_ok = 0;
	return SEPDEV_OK;
}

extern "C" sepb *sepb_create_typed(int nsys, const int *npart, const double *L, double skin, double dt,
				   int ntypes, const double *ljparams)
{
	if (ntypes < 1 || ntypes > SEPB_MAXTYPES || !ljparams) {
		batch_fail("sepb_create_typed: 1 to 4 types and their parameters are required", SEPDEV_EINVAL);
		return NULL;
	}
	double rc = 0.0;
	const double *p0 = NULL;
	for (int a = 0; a < ntypes; a++)
		for (int c = 0; c < ntypes; c++) {
			const double *p = ljparams + 4 * (a * ntypes + c), *q = ljparams + 4 * (c * ntypes + a);
			if (p[0] != q[0] || p[1] != q[1] || p[2] != q[2] || p[3] != q[3]) {
				batch_fail("sepb_create_typed: the parameters of a type pair must not depend on its order",
					   SEPDEV_EINVAL);
				return NULL;
			}
			if (p[1] == 0.0) continue;
			if (!(p[0] > 0) || !(p[2] > 0)) {
				batch_fail("sepb_create_typed: cut-off and sigma must be positive", SEPDEV_EINVAL);
				return NULL;
			}
			if (p[0] > rc) rc = p[0];
			if (!p0) p0 = p;
		}
	if (!p0) {
		batch_fail("sepb_create_typed: no type pair interacts", SEPDEV_EINVAL);
		return NULL;
	}
	sepb *b = batch_make(nsys, npart, L, rc, skin, dt, p0, 1);
	if (!b) return NULL;
	b->ntypes = ntypes;
	memcpy(b->tparam, ljparams, sizeof(double) * 4 * ntypes * ntypes);
	// the parameter table, unscaled: every pair's own cut-off and shift
	sepdev_pairset ps;
	memset(&ps, 0, sizeof ps);
	ps.ntypes = ntypes;
	for (int k = 0; k < ntypes * ntypes; k++) {
		const double *p = ljparams + 4 * k;
		sepdev_pot &P = ps.pot[k];
		P.kind = SEPDEV_POT_LJ;
		if (p[1] == 0.0) continue;           // no term: rc2 = 0, eps = 0
		P.rc2 = (float)(p[0] * p[0]);
		P.eps48 = (float)(48.0 * p[1]);
		P.eps4 = (float)(4.0 * p[1]);
		P.sig2 = (float)(p[2] * p[2]);
		P.aw = (float)p[3];
		P.awh = (float)(0.5 * p[3]);
		P.ushift = (float)(-4.0 * p[1] * (pow(p[2] / p[0], 12.) - p[3] * pow(p[2] / p[0], 6.)));
	}
	int rc0 = sepdev_upload_pairset(b->d, &ps);
	if (!rc0) rc0 = cudaStreamSynchronize(b->d->st) == cudaSuccess ? SEPDEV_OK : SEPDEV_ECUDA;
	if (rc0) {
		sepb_destroy(b);
		return NULL;
	}
	return b;
}

extern "C" int sepb_set_types(sepb *b, int s, const int *type)
{
	if (!b || s < 0 || s >= b->nsys || !type) return batch_fail("sepb_set_types: invalid arguments", SEPDEV_EINVAL);
	if (!b->fresh[s])
		return batch_fail("sepb_set_types: call it after sepb_set_state of the system, before a run",
				  SEPDEV_EINVAL);
	const BatchSys &S = b->hsys[s];
	sepdev *d = b->d;
	std::vector<int4> hp(S.npad);
	CK(cudaMemcpy(hp.data(), d->pos[0] + S.off, sizeof(int4) * S.npad, cudaMemcpyDeviceToHost));
	for (int i = 0; i < S.n; i++) {
		if (type[i] < 0 || type[i] >= b->ntypes)
			return batch_fail("sepb_set_types: type id outside 0..ntypes-1", SEPDEV_EINVAL);
		hp[i].w = type[i];           // slots are in the system's own order until its first run
	}
	CK(cudaMemcpy(d->pos[0] + S.off, hp.data(), sizeof(int4) * S.npad, cudaMemcpyHostToDevice));
	CK(cudaMemcpy(d->pos[1] + S.off, hp.data(), sizeof(int4) * S.npad, cudaMemcpyHostToDevice));
	return SEPDEV_OK;
}

extern "C" int sepb_set_thermostat(sepb *b, const double *T0, double tau, const double *alpha)
{
	if (!b) return batch_fail("sepb_set_thermostat: no batch", SEPDEV_EINVAL);
	if (!T0) { b->nh = 0; return SEPDEV_OK; }
	if (!(tau > 0)) return batch_fail("sepb_set_thermostat: tau must be positive", SEPDEV_EINVAL);
	b->nh = 1;
	b->tau = tau;
	for (int s = 0; s < b->nsys; s++) {
		b->hsys[s].T0 = T0[s];
		b->alpha0[s] = alpha ? alpha[s] : 0.0;
		b->h_bs[s].alpha_last = b->alpha0[s];
	}
	CK(cudaMemcpy(b->sys, b->hsys.data(), sizeof(BatchSys) * b->nsys, cudaMemcpyHostToDevice));
	return SEPDEV_OK;
}

PairArgs batch_pair_args(sepb *b, int parity)
{
	sepdev_pairset ps;
	memset(&ps, 0, sizeof ps);
	ps.ntypes = 1;
	sepdev_pot &P = ps.pot[0];
	P.kind = SEPDEV_POT_LJ;
	P.rc2 = (float)(b->cf * b->cf);
	P.eps48 = (float)(48.0 * b->eps);
	P.eps4 = (float)(4.0 * b->eps);
	P.sig2 = (float)(b->sigma * b->sigma);
	P.aw = (float)b->aw;
	P.awh = (float)(0.5 * b->aw);
	P.ushift = (float)b->ushift;
	P.ushl = (float)(b->ushift - (double)P.ushift);
	PairArgs a;
	sepdev_fill_args(b->d, a, &ps, b->dt, b->nh, 0.0, 0, 0, 0, parity);
	a.flags = b->d->flags;
	return a;
}

BatchDecide batch_decide_args(sepb *b)
{
	BatchDecide a;
	memset(&a, 0, sizeof a);
	a.sys = b->sys;
	a.bs = b->bs;
	a.run = b->run;
	a.slots = b->slots;
	a.flag = b->flag;
	a.oflow = b->d->flags;
	a.nsys = b->nsys;
	a.thr2 = (float)(0.25 * b->skin * b->skin);
	a.dt_tau2 = b->dt / (b->tau * b->tau);
	a.nh = b->nh;
	return a;
}

static BGather gather_args(sepb *b, int parity)
{
	sepdev *d = b->d;
	BGather g;
	g.sys = b->sys; g.wsys = b->wsys; g.flag = b->flag; g.nwarps = b->nwarps;
	g.perm = d->perm;
	g.pos = d->pos[parity]; g.pos_o = d->pos[parity ^ 1];
	g.xlo = d->xlo; g.xlo_o = d->xlo_b;
	g.vhi = d->vhi; g.vhi_o = d->vhi_b;
	g.vlo = d->vlo; g.vlo_o = d->vlo_b;
	g.frc = d->frc; g.frc_o = d->frc_b;
	g.cross = d->cross; g.cross_o = d->cross_b;
	g.cbase = d->cbase; g.cbase_o = d->cbase_b;
	g.gid = d->gid; g.gid_o = d->gid_b;
	g.xn = d->xn; g.inv = d->inv;
	return g;
}

// sort + list build of the flagged systems from buffer `parity`; capturable
// cell lists of the flagged systems without moving particles: bin, scan,
// scatter of slot indices, deterministic order inside cells; capturable
int batch_cells_launch(sepb *b, int parity)
{
	sepdev *d = b->d;
	const int B = 256;
	const long nt = b->ntot;
	CK(cudaMemsetAsync(b->cellcount, 0, sizeof(int) * b->ncells, d->st));
	kb_bin<<<grid_for(nt, B), B, 0, d->st>>>(b->sys, b->wsys, b->nwarps, b->flag, d->pos[parity],
						d->cellof, d->celloff, b->cellcount);
	kb_scan<<<b->nsys, 256, 0, d->st>>>(b->sys, b->flag, b->cellcount, b->cellstart);
	kb_scatter<<<grid_for(nt, B), B, 0, d->st>>>(b->wsys, b->nwarps, b->flag, d->cellof, d->celloff,
						    b->cellstart, d->perm);
	kb_cellsort<<<grid_for(b->ncells * 32, B), B, 0, d->st>>>(b->ncells, b->csys, b->flag, b->cellstart,
								 d->gid, d->pos[parity], d->perm);
	CKL(d);
	return SEPDEV_OK;
}

int batch_rebuild_launch(sepb *b, int parity)
{
	sepdev *d = b->d;
	const int B = 256;
	const long nt = b->ntot;
	CK(cudaMemsetAsync(b->cellcount, 0, sizeof(int) * b->ncells, d->st));
	kb_bin<<<grid_for(nt, B), B, 0, d->st>>>(b->sys, b->wsys, b->nwarps, b->flag, d->pos[parity],
						d->cellof, d->celloff, b->cellcount);
	kb_scan<<<b->nsys, 256, 0, d->st>>>(b->sys, b->flag, b->cellcount, b->cellstart);
	kb_scatter<<<grid_for(nt, B), B, 0, d->st>>>(b->wsys, b->nwarps, b->flag, d->cellof, d->celloff,
						    b->cellstart, d->perm);
	kb_cellsort<<<grid_for(b->ncells * 32, B), B, 0, d->st>>>(b->ncells, b->csys, b->flag, b->cellstart,
								 d->gid, d->pos[parity], d->perm);
	BGather g = gather_args(b, parity);
	kb_gather<<<grid_for(nt, B), B, 0, d->st>>>(g);
	kb_copyback<<<grid_for(nt, B), B, 0, d->st>>>(g);
	CK(cudaMemsetAsync(b->fcnt, 0, sizeof(int), d->st));
	kb_compact<<<b->nsys, 128, 0, d->st>>>(b->sys, b->flag, b->fw, b->fcnt);
	CKL(d);
	CK(cudaMemsetAsync(d->flags, 0, sizeof(unsigned) * 2, d->st));
	return sepdev_batch_build(d, parity, b->cellstart, b->sys, b->wsys, b->nwarps, b->flag,
				  (float)((b->rc + b->skin) * (b->rc + b->skin)), NULL, b->fw, b->fcnt);
}

int batch_step_launch(sepb *b, int parity, const BatchDecide &dec)
{
	PairArgs a = batch_pair_args(b, parity);
	CK(cudaGetLastError());
	int rc = sepdev_batch_step(b->d, a, b->sys, b->wstep, b->nstepw, b->bs, b->run, b->slots, dec,
				   b->ntypes > 1);
	if (rc) return rc;
	kb_decide<<<grid_for((long)b->nsys * 32, 256), 256, 0, b->d->st>>>(dec);
	CKL(b->d);
	return SEPDEV_OK;
}

static int capture_tail(sepdev *d, cudaGraphNode_t *out)
{
	cudaStreamCaptureStatus st;
	const cudaGraphNode_t *deps = NULL;
	size_t nd = 0;
	cudaError_t e = cudaStreamGetCaptureInfo(d->st, &st, NULL, NULL, &deps, NULL, &nd);
	if (e != cudaSuccess || nd != 1) { sepdev_set_error("capture info", e); return SEPDEV_ECUDA; }
	*out = deps[0];
	return SEPDEV_OK;
}

static int build_graph(sepb *b, int parity)
{
	sepdev *d = b->d;
	if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = NULL; }
	if (b->graph) { cudaGraphDestroy(b->graph); b->graph = NULL; }
	CK(cudaGraphCreate(&b->graph, 0));
	cudaGraphConditionalHandle hw, hif[RUN_UNROLL_B];
	CK(cudaGraphConditionalHandleCreate(&hw, b->graph, 1, cudaGraphCondAssignDefault));
	for (int k = 0; k < RUN_UNROLL_B; k++)
		CK(cudaGraphConditionalHandleCreate(&hif[k], b->graph, 0, cudaGraphCondAssignDefault));
	cudaGraphNodeParams wp = {cudaGraphNodeTypeConditional};
	wp.conditional.handle = hw;
	wp.conditional.type = cudaGraphCondTypeWhile;
	wp.conditional.size = 1;
	cudaGraphNode_t wnode;
	CK(cudaGraphAddNode(&wnode, b->graph, NULL, NULL, 0, &wp));
	cudaGraph_t body = wp.conditional.phGraph_out[0];
	cudaGraphNode_t tail = NULL;
	for (int k = 0; k < RUN_UNROLL_B; k++) {
		const int p = parity ^ (k & 1);
		cudaGraphNodeParams ip = {cudaGraphNodeTypeConditional};
		ip.conditional.handle = hif[k];
		ip.conditional.type = cudaGraphCondTypeIf;
		ip.conditional.size = 1;
		cudaGraphNode_t nif;
		CK(cudaGraphAddNode(&nif, body, k ? &tail : NULL, NULL, k ? 1 : 0, &ip));
		CK(cudaStreamBeginCaptureToGraph(d->st, ip.conditional.phGraph_out[0], NULL, NULL, 0,
						 cudaStreamCaptureModeRelaxed));
		int rc = batch_rebuild_launch(b, p);
		cudaGraph_t tmp;
		cudaError_t e = cudaStreamEndCapture(d->st, &tmp);
		if (rc) return rc;
		if (e != cudaSuccess) { sepdev_set_error("capture(batch rebuild)", e); return SEPDEV_ECUDA; }
		BatchDecide dec = batch_decide_args(b);
		dec.use_handles = 1;
		dec.h_next = hif[(k + 1) % RUN_UNROLL_B];
		dec.h_while = hw;
		dec.reset_while = (k == 0);
		dec.pair_end = (k == RUN_UNROLL_B - 1);
		CK(cudaStreamBeginCaptureToGraph(d->st, body, &nif, NULL, 1, cudaStreamCaptureModeRelaxed));
		rc = batch_step_launch(b, p, dec);
		if (!rc) rc = capture_tail(d, &tail);
		e = cudaStreamEndCapture(d->st, &tmp);
		if (rc) return rc;
		if (e != cudaSuccess) { sepdev_set_error("capture(batch step)", e); return SEPDEV_ECUDA; }
	}
	CK(cudaGraphInstantiate(&b->exec, b->graph, 0));
	b->graph_parity = parity;
	b->graph_nl = d->nl;
	b->graph_maxnb = d->maxnb;
	return SEPDEV_OK;
}

// upload the per-system state, with alpha advanced for the first step
// exactly as sep_gpu_run / sep_nosehoover do on the host
static int run_begin(sepb *b, long nsteps)
{
	for (int s = 0; s < b->nsys; s++) {
		BatchState &st = b->h_bs[s];
		double a = st.alpha_last;
		if (b->nh) {
			const double ekin = 0.5 * st.sumv2 / b->hsys[s].n;
			const double temp = 0.666667 * ekin;
			a = a + b->dt / (b->tau * b->tau) * (temp / b->hsys[s].T0 - 1.0);
		}
		st.alpha = a;
		st.alpha_last = a;
		st.ntrig = 0;
	}
	BatchRun &r = *b->h_run;
	r.remaining = 0;
	r.done = 0;
	r.total = nsteps;
	r.arrive = 0;
	r.any = 0;
	r.abort = 0;
	sepdev *d = b->d;
	CK(cudaMemcpyAsync(b->bs, b->h_bs, sizeof(BatchState) * b->nsys, cudaMemcpyHostToDevice, d->st));
	CK(cudaMemcpyAsync(b->run, b->h_run, sizeof(BatchRun), cudaMemcpyHostToDevice, d->st));
	CK(cudaMemsetAsync(b->slots, 0, sizeof(long long) * SLOT_FIELDS * b->nsys, d->st));
	CK(cudaMemsetAsync(d->flags, 0, sizeof(unsigned) * 2, d->st));
	return SEPDEV_OK;
}

int batch_initial_lists(sepb *b)
{
	sepdev *d = b->d;
	std::vector<unsigned> ones(b->nsys, 1u);
	CK(cudaMemcpyAsync(b->flag, ones.data(), sizeof(unsigned) * b->nsys, cudaMemcpyHostToDevice, d->st));
	int rc = batch_rebuild_launch(b, d->cur);
	if (rc) return rc;
	unsigned fl[2];
	CK(cudaMemcpyAsync(fl, d->flags, sizeof fl, cudaMemcpyDeviceToHost, d->st));
	CK(cudaMemsetAsync(b->flag, 0, sizeof(unsigned) * b->nsys, d->st));
	CK(cudaStreamSynchronize(d->st));
	if (fl[0] & 1u) {
		// the first lists set the capacity: grow once to their largest count
		if ((rc = sepdev_grow_list_to(d, (int)(fl[1] + fl[1] / 2 + 32)))) return rc;
		CK(cudaMemcpyAsync(b->flag, ones.data(), sizeof(unsigned) * b->nsys, cudaMemcpyHostToDevice, d->st));
		if ((rc = batch_rebuild_launch(b, d->cur))) return rc;
		CK(cudaMemcpyAsync(fl, d->flags, sizeof fl, cudaMemcpyDeviceToHost, d->st));
		CK(cudaMemsetAsync(b->flag, 0, sizeof(unsigned) * b->nsys, d->st));
		CK(cudaStreamSynchronize(d->st));
		if (fl[0] & 1u) return batch_fail("sepb: neighbour list overflow at set-up", SEPDEV_EOVERFLOW);
	}
	b->list_ok = 1;
	b->h_run->last_any = 0;
	for (int s = 0; s < b->nsys; s++) b->fresh[s] = 0;
	return SEPDEV_OK;
}

static int run_steps(sepb *b, long nsteps, int timed, long flush, double *ms)
{
	if (!b || nsteps < 0) return batch_fail("sepb_run: invalid arguments", SEPDEV_EINVAL);
	for (int s = 0; s < b->nsys; s++)
		if (!b->have[s]) return batch_fail("sepb_run: a system has no state (sepb_set_state)", SEPDEV_EINVAL);
	sepdev *d = b->d;
	int rc;
	if (!b->list_ok && (rc = batch_initial_lists(b))) return rc;
	if (nsteps == 0) return SEPDEV_OK;
	const unsigned pending = b->h_run->last_any;
	if ((rc = run_begin(b, nsteps))) return rc;
	BatchRun *h = b->h_run;
	// a rebuild the previous step asked for runs before the next step; inside
	// a graph the decisions set the IF nodes, across launches the host does it
	h->last_any = pending;
	float total_ms = 0.f;
	cudaEvent_t e0 = d->ev[6], e1 = d->ev[7];
	while (h->done < nsteps) {
		const long todo = nsteps - h->done;
		const long done0 = h->done;
		if (timed) {
			// one step per span, the L2 flushed before it outside the span
			if (flush > 0) {
				if (!b->flush_buf || b->flush_bytes < (size_t)flush) {
					if (b->flush_buf) cudaFree(b->flush_buf);
					b->flush_buf = NULL;
					CK(cudaMalloc(&b->flush_buf, (size_t)flush));
					b->flush_bytes = (size_t)flush;
				}
				kb_flush<<<d->nsm * 4, 512, 0, d->st>>>((uint4 *)b->flush_buf, flush / 16, (unsigned)done0);
			}
			CK(cudaEventRecord(e0, d->st));
			if (h->last_any && (rc = batch_rebuild_launch(b, d->cur))) return rc;
			if ((rc = batch_step_launch(b, d->cur, batch_decide_args(b)))) return rc;
			CK(cudaEventRecord(e1, d->st));
		} else if (todo >= RUN_UNROLL_B) {
			if (h->last_any && (rc = batch_rebuild_launch(b, d->cur))) return rc;
			h->remaining = todo / RUN_UNROLL_B;
			CK(cudaMemcpyAsync(b->run, h, sizeof *h, cudaMemcpyHostToDevice, d->st));
			const bool stale = !b->exec || b->graph_parity != d->cur || b->graph_nl != d->nl ||
					   b->graph_maxnb != d->maxnb;
			if (stale && (rc = build_graph(b, d->cur))) return rc;
			CK(cudaGraphLaunch(b->exec, d->st));
		} else {
			if (h->last_any && (rc = batch_rebuild_launch(b, d->cur))) return rc;
			if ((rc = batch_step_launch(b, d->cur, batch_decide_args(b)))) return rc;
		}
		CK(cudaMemcpyAsync(h, b->run, sizeof *h, cudaMemcpyDeviceToHost, d->st));
		CK(cudaStreamSynchronize(d->st));
		if (timed) {
			float x = 0.f;
			CK(cudaEventElapsedTime(&x, e0, e1));
			total_ms += x;
		}
		if ((h->done - done0) & 1) d->cur ^= 1;
		if (h->abort) return batch_fail("sepb_run: neighbour list overflow", SEPDEV_EOVERFLOW);
	}
	CK(cudaMemcpy(b->h_bs, b->bs, sizeof(BatchState) * b->nsys, cudaMemcpyDeviceToHost));
	for (int s = 0; s < b->nsys; s++) b->nupd[s] += (unsigned)b->h_bs[s].ntrig;
	if (ms) *ms = total_ms;
	return SEPDEV_OK;
}

extern "C" int sepb_run(sepb *b, long nsteps)
{
	return run_steps(b, nsteps, 0, 0, NULL);
}

extern "C" int sepb_run_timed(sepb *b, long nsteps, long flush_bytes, double *ms_steps)
{
	return run_steps(b, nsteps, 1, flush_bytes, ms_steps);
}

extern "C" int sepb_get_state(sepb *b, int s, double *x, double *v, double *f)
{
	if (!b || s < 0 || s >= b->nsys) return batch_fail("sepb_get_state: invalid arguments", SEPDEV_EINVAL);
	const BatchSys &S = b->hsys[s];
	sepdev *d = b->d;
	const int n = S.n;
	std::vector<int4> hp(n);
	std::vector<uint4> hl(n);
	std::vector<float4> hvh(n), hvl(n), hf(n);
	std::vector<int> hg(n);
	const size_t o = (size_t)S.off;
	CK(cudaStreamSynchronize(d->st));
	CK(cudaMemcpy(hp.data(), d->pos[d->cur] + o, sizeof(int4) * n, cudaMemcpyDeviceToHost));
	CK(cudaMemcpy(hl.data(), d->xlo + o, sizeof(uint4) * n, cudaMemcpyDeviceToHost));
	CK(cudaMemcpy(hvh.data(), d->vhi + o, sizeof(float4) * n, cudaMemcpyDeviceToHost));
	CK(cudaMemcpy(hvl.data(), d->vlo + o, sizeof(float4) * n, cudaMemcpyDeviceToHost));
	CK(cudaMemcpy(hf.data(), d->frc + o, sizeof(float4) * n, cudaMemcpyDeviceToHost));
	CK(cudaMemcpy(hg.data(), d->gid + o, sizeof(int) * n, cudaMemcpyDeviceToHost));
	// the padding sits at the end of the system's slots, so the first n
	// slots hold exactly its particles
	for (int t = 0; t < n; t++) {
		const int u = hg[t];
		if (u < 0 || u >= n) return batch_fail("sepb_get_state: slot map corrupt", SEPDEV_EINVAL);
		const unsigned hi[3] = {(unsigned)hp[t].x, (unsigned)hp[t].y, (unsigned)hp[t].z};
		const unsigned lo[3] = {hl[t].x, hl[t].y, hl[t].z};
		const float vh[3] = {hvh[t].x, hvh[t].y, hvh[t].z}, vl[3] = {hvl[t].x, hvl[t].y, hvl[t].z};
		const float ff[3] = {hf[t].x, hf[t].y, hf[t].z};
		for (int k = 0; k < 3; k++) {
			if (x) x[3 * u + k] = batch_from_fixed(hi[k], lo[k], S.L);
			if (v) v[3 * u + k] = (double)vh[k] + (double)vl[k];
			if (f) f[3 * u + k] = (double)ff[k];
		}
	}
	return SEPDEV_OK;
}

extern "C" int sepb_get_results(sepb *b, sepb_result *out)
{
	if (!b || !out) return batch_fail("sepb_get_results: invalid arguments", SEPDEV_EINVAL);
	const int map[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
	for (int s = 0; s < b->nsys; s++) {
		const BatchState &st = b->h_bs[s];
		sepb_result &r = out[s];
		r.epot = st.last[SLOT_EPOT0];
		r.ekin = 0.5 * st.last[SLOT_EKIN];
		for (int k = 0; k < 3; k++)
			for (int kk = 0; kk < 3; kk++) {
				r.pot_P[k][kk] = st.last[SLOT_POTP + map[k][kk]];
				r.kin_P[k][kk] = st.last[SLOT_KINP + map[k][kk]];
			}
		r.alpha = st.alpha_last;
		r.max_dist2 = st.last[SLOT_MAXD2];
		r.nupdate = b->nupd[s];
		r.sumv2 = st.sumv2;
	}
	return SEPDEV_OK;
}

extern "C" long sepb_particles(const sepb *b) { return b ? b->ntot : -1; }
