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
//   4. k_cellsort particles of a cell ordered by x (ties by user index), so
//                 a run of particles is a compact slab along the cell row and
//                 the order, and every floating-point sum after it, are
//                 run-to-run identical;
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
#include "dev_batch.cuh"
#include "dev_cellsort.cuh"

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

// exclusive scan of count[0..m) into start[0..m] (start[m] = total), one
// block of 1024 threads.  The counts are taken in tiles of 1024 * SCAN_REG:
// each thread owns SCAN_REG consecutive counts (16-byte loads and stores),
// sums them serially, and one block-wide scan of the thread sums (warp
// shuffles plus a pass over the 32 warp totals) gives every thread its
// offset; the running total carries from tile to tile.
#define SCAN_REG 16
__global__ void __launch_bounds__(1024) k_scan(long m, const int *__restrict__ count, int *__restrict__ start)
{
	__shared__ int wsum[32];
	const unsigned FULL = 0xffffffffu;
	const int t = threadIdx.x, lane = t & 31, w = t >> 5;
	int carry = 0;
	for (long base = 0; base < m; base += 1024L * SCAN_REG) {
		const long k0 = base + (long)t * SCAN_REG;
		int v[SCAN_REG];
		if (k0 + SCAN_REG <= m) {
			const int4 *src = (const int4 *)(count + k0);
#pragma unroll
			for (int q = 0; q < SCAN_REG / 4; q++) {
				const int4 c = __ldg(src + q);
				v[4 * q] = c.x; v[4 * q + 1] = c.y; v[4 * q + 2] = c.z; v[4 * q + 3] = c.w;
			}
		} else {
#pragma unroll
			for (int r = 0; r < SCAN_REG; r++) v[r] = k0 + r < m ? __ldg(count + k0 + r) : 0;
		}
		int sum = 0;
#pragma unroll
		for (int r = 0; r < SCAN_REG; r++) { const int c = v[r]; v[r] = sum; sum += c; }
		int x = sum;
#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			const int y = __shfl_up_sync(FULL, x, o);
			if (lane >= o) x += y;
		}
		if (lane == 31) wsum[w] = x;
		__syncthreads();
		if (w == 0) {
			int ws = wsum[lane];
#pragma unroll
			for (int o = 1; o < 32; o <<= 1) {
				const int y = __shfl_up_sync(FULL, ws, o);
				if (lane >= o) ws += y;
			}
			wsum[lane] = ws;                            // inclusive over warps
		}
		__syncthreads();
		const int off = carry + (w ? wsum[w - 1] : 0) + x - sum;
		const int total = wsum[31];
		if (k0 + SCAN_REG <= m) {
			int4 *dst = (int4 *)(start + k0);
#pragma unroll
			for (int q = 0; q < SCAN_REG / 4; q++)
				dst[q] = make_int4(off + v[4 * q], off + v[4 * q + 1], off + v[4 * q + 2], off + v[4 * q + 3]);
		} else {
#pragma unroll
			for (int r = 0; r < SCAN_REG; r++)
				if (k0 + r < m) start[k0 + r] = off + v[r];
		}
		carry += total;
		__syncthreads();                                    // wsum is reused by the next tile
	}
	if (t == 0) start[m] = carry;
}

__global__ void k_scatter(long n, const int *__restrict__ cellof, const int *__restrict__ celloff,
			  const int *__restrict__ start, int *__restrict__ perm)
{
	long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
	if (s < n) perm[start[cellof[s]] + celloff[s]] = (int)s;
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
	const float4 *ext[SEPDEV_NEXT]; float4 *ext_o[SEPDEV_NEXT];
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
#pragma unroll
	for (int k = 0; k < SEPDEV_NEXT; k++)
		if (a.ext[k]) a.ext_o[k][t] = a.ext[k][o];
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
	const int *perm;        // PERM builds: the cell lists hold slot indices (particles not moved)
};

// Tile-staged list build: one warp per tile of 32 consecutive particles (in
// cell order a tile covers a short run of cells along x).  For each row run
// of the tile the warp stages the candidates of the deduplicated 3x3
// neighbouring rows over the x range [first cell - 1, last cell + 1] with
// coalesced loads (a cell row is one contiguous range of the sorted
// particles), converted once into FP32 offsets from the run's first
// particle; candidates farther than rlist from the bounding box of the run's
// particles are dropped and the rest compacted into shared memory, where
// every lane of the run tests them (broadcast reads).  Candidates outside a
// lane's own 27 cells are at least one cell edge (>= rlist) away and fail the
// distance test.
// Accepted entries go to a per-warp shared ring of BT_RING rows ([row][lane],
// conflict-free) with a branch-free append; complete four-entry groups are
// written out as 16-byte stores whenever the next chunk could wrap the ring
// onto entries not yet written.
#define BT_WARPS 4
#define BT_CAP 32      // staged candidates per chunk
#define BT_RING 64     // ring rows per warp (power of two)

__device__ __forceinline__ int wrapc(int c, int n) { return c < 0 ? c + n : (c >= n ? c - n : c); }

__device__ __forceinline__ float warp_min_f(float v, unsigned mask)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(mask, v, o));
	return v;
}

__device__ __forceinline__ float warp_max_f(float v, unsigned mask)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(mask, v, o));
	return v;
}

// One warp builds the lists of the tile of 32 particles starting at i0 (n:
// end of the particles to build); sp and ring are the warp's shared staging.
// WRAPFAST: runs whose region wraps around the box (small boxes: the batched
// systems) also get the branch-free test loop; without it they take the
// general loop, which keeps the common in-box loop's code tight.
// MOLX (same-molecule exclusions): the candidates' molecule indices are
// staged in spm beside their positions, and in-box runs take a branch-free
// loop that tests them from shared memory.
// PERM: the particles are not in cell order; a cell's members are the
// slots perm[cellstart[c] .. cellstart[c + 1]) (the adjoint's fixed slots).
// TB = 2: two lanes per particle, a tile of 16 particles per warp (twice
// the warps, for systems too small to fill the GPU).  Lane p (p < 16) and
// lane p + 16 hold particle i0 + p and split every staged chunk: lane p
// tests its first half, lane p + 16 the second half into spare rows of its
// own column, and lane p then appends those hits after its own.  A
// particle's list is therefore the same, entry for entry, as with one lane.
template <bool WRAPFAST, bool MOLX = false, bool PERM = false, int TB = 1>
__device__ __forceinline__ void build_tile(long n, const BuildArgs &a, long i0, float4 *sp, int *ring,
					   int *spm = nullptr)
{
	static_assert(TB == 1 || TB == 2, "one or two lanes per particle");
	const unsigned FULL = 0xffffffffu;
	const int lane = threadIdx.x & 31;
	const int hh = TB == 2 ? lane >> 4 : 0;          // which half of the particle's lane pair
	if (i0 >= n) return;
	const long i = i0 + (TB == 2 ? (lane & 15) : lane);
	const bool act = i < n;
	const bool own = act && hh == 0;                   // the lane that writes the particle's list
	const int4 pi = a.pos[act ? i : i0];
	const int nc0 = a.nc[0], nc1 = a.nc[1], nc2 = a.nc[2];
	const int cx = (int)__umulhi((unsigned)pi.x, (unsigned)nc0);
	const int cy = (int)__umulhi((unsigned)pi.y, (unsigned)nc1);
	const int cz = (int)__umulhi((unsigned)pi.z, (unsigned)nc2);
	const int row = cy + nc1 * cz;
	// TB = 2: lane l also holds particle l of the parent tile (the 32
	// particles one lane per particle would take), whose run in a row fixes
	// the staged segments, their order, the frame of the offsets and the
	// in-box test exactly as with one lane per particle
	int4 ppi = pi;
	int pcx = cx, prow = row;
	bool pact = act;
	if (TB == 2) {
		const long P = (i0 & ~31L) + lane;
		pact = P < n;
		ppi = a.pos[pact ? P : i0];
		pcx = (int)__umulhi((unsigned)ppi.x, (unsigned)nc0);
		prow = (int)__umulhi((unsigned)ppi.y, (unsigned)nc1) +
		       nc1 * (int)__umulhi((unsigned)ppi.z, (unsigned)nc2);
	}
	int4 *gbase = (int4 *)(a.nl + nl_index(i, 0, a.maxnb));   // this lane's group 0
	const int gi = act ? a.gid[i] : -1, mi = act ? a.mol[i] : -1;
	const int lo1 = nc1 >= 3 ? -1 : 0, hi1 = nc1 >= 2 ? 1 : 0;
	const int lo2 = nc2 >= 3 ? -1 : 0, hi2 = nc2 >= 2 ? 1 : 0;
	const int cap = a.maxnb;
	const float rl = sqrtf(a.rl2), rlm = rl * 1.0001f;
	int cnt = 0, flushed = 0;     // entries found / entries written out (multiple of 4)
	bool me = false, local = false;
	float mx = 0.f, my = 0.f, mz = 0.f;
	float bx0 = 0.f, bx1 = 0.f, by0 = 0.f, by1 = 0.f, bz0 = 0.f, bz1 = 0.f;
	int4 ref = pi;
	auto excluded = [&](int j) -> bool {
		if (a.excl == SEPDEV_EXCL_SAMEMOL) return mi != -1 && mi == a.mol[j];
		const int gj = a.gid[j];
		return in_csr(a.exs, a.exi, gi, gj) || in_csr(a.exs, a.exi, gj, gi);
	};
	auto flush = [&]() {
		const int top = cnt < cap ? cnt : cap;
		const int g0 = flushed >> 2, g1 = (top + 3) >> 2;
		const int gmin = __reduce_min_sync(FULL, own ? g0 : 0x7fffffff);
		const int gmax = __reduce_max_sync(FULL, own ? g1 : 0);
		for (int g = gmin; g < gmax; g++) {
			if (own && g >= g0 && g < g1) {
				const int r = (4 * g) & (BT_RING - 1), b0 = 4 * g;
				// a group past the count is padded with the particle itself
				// (separation zero), so readers take whole groups of four
				gbase[g * 32] = make_int4(ring[r * 32 + lane],
							  b0 + 1 < top ? ring[(r + 1) * 32 + lane] : (int)i,
							  b0 + 2 < top ? ring[(r + 2) * 32 + lane] : (int)i,
							  b0 + 3 < top ? ring[(r + 3) * 32 + lane] : (int)i);
			}
		}
		flushed = top & ~3;
	};
	// 0 < r^2 < rlist^2 as one unsigned comparison of the bit patterns
	// (r^2 >= 0): the zero separation of a particle with itself fails it,
	// so the fast loops need no index test
	const unsigned rl2m1 = __float_as_uint(a.rl2) - 1u;
	auto inlist = [&](float r2) { return (__float_as_uint(r2) - 1u) < rl2m1; };
	auto test = [&](int fill) {
		__syncwarp();
		// entries not yet written out must stay in the ring through this chunk
		const int span = __reduce_max_sync(FULL, own ? cnt - flushed : 0);
		if (span + fill > BT_RING) flush();
		// this lane's share of the chunk, and where its hits go: after the
		// particle's entries, or (second lane of a pair) from row 0 of its
		// own column, which holds no particle's entries
		int c0 = 0, c1 = fill, w = cnt;
		if (TB == 2) {
			const int half = (fill + 1) >> 1;
			c0 = hh ? half : 0;
			c1 = hh ? fill : half;
			w = hh ? 0 : cnt;
		}
		if (me) {
			if (MOLX && local) {
#pragma unroll 4
				for (int c = c0; c < c1; c++) {
					const float4 q = sp[c];
					const float dx = mx - q.x, dy = my - q.y, dz = mz - q.z;
					const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
					const int j = __float_as_int(q.w);
					const bool hit = inlist(r2) & !((mi != -1) & (mi == spm[c]));
					ring[(w & (BT_RING - 1)) * 32 + lane] = j;
					w += hit ? 1 : 0;
				}
			} else if (local && a.excl == SEPDEV_EXCL_NONE) {
#pragma unroll 4
				for (int c = c0; c < c1; c++) {
					const float4 q = sp[c];
					const float dx = mx - q.x, dy = my - q.y, dz = mz - q.z;
					const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
					const int j = __float_as_int(q.w);
					const bool hit = inlist(r2);
					ring[(w & (BT_RING - 1)) * 32 + lane] = j;
					w += hit ? 1 : 0;
				}
			} else if (WRAPFAST && a.excl == SEPDEV_EXCL_NONE) {
				// minimum-image separations per candidate, appended in
				// candidate order without branches (as the local form)
#pragma unroll 4
				for (int c = c0; c < c1; c++) {
					const float4 q = sp[c];
					const float dx = sep_hi(pi.x, __float_as_int(q.x), a.fs[0]);
					const float dy = sep_hi(pi.y, __float_as_int(q.y), a.fs[1]);
					const float dz = sep_hi(pi.z, __float_as_int(q.z), a.fs[2]);
					const int j = __float_as_int(q.w);
					const bool hit = inlist(dx * dx + dy * dy + dz * dz);
					ring[(w & (BT_RING - 1)) * 32 + lane] = j;
					w += hit ? 1 : 0;
				}
			} else {
				for (int c = c0; c < c1; c++) {
					const float4 q = sp[c];
					const int j = __float_as_int(q.w);
					float dx, dy, dz;
					if (local) { dx = mx - q.x; dy = my - q.y; dz = mz - q.z; }
					else {
						dx = sep_hi(pi.x, __float_as_int(q.x), a.fs[0]);
						dy = sep_hi(pi.y, __float_as_int(q.y), a.fs[1]);
						dz = sep_hi(pi.z, __float_as_int(q.z), a.fs[2]);
					}
					if (!(dx * dx + dy * dy + dz * dz < a.rl2) || j == (int)i) continue;
					if (a.excl != SEPDEV_EXCL_NONE && excluded(j)) continue;
					ring[(w & (BT_RING - 1)) * 32 + lane] = j;
					w++;
				}
			}
		}
		if (TB == 1 || hh == 0) cnt = w;
		if (TB == 2) {
			// the second lane's hits follow the first lane's, in chunk order
			__syncwarp();
			const int m = __shfl_down_sync(FULL, me && hh ? w : 0, 16);
			if (me && hh == 0)
				for (int k = 0; k < m; k++, cnt++)
					ring[(cnt & (BT_RING - 1)) * 32 + lane] = ring[k * 32 + lane + 16];
		}
		__syncwarp();
	};
	unsigned todo = __ballot_sync(FULL, act);
	while (todo) {
		const int leader = __ffs(todo) - 1;
		const int rrow = __shfl_sync(FULL, row, leader);
		const unsigned mine = __ballot_sync(FULL, act && row == rrow);
		todo &= ~mine;
		me = (mine >> lane) & 1u;
		// the run's cells along x: in cell order its first and last lanes;
		// over index-only cell lists the lanes are in no order (min, max)
		const unsigned pm = TB == 2 ? __ballot_sync(FULL, pact && prow == rrow) : mine;
		const int xlo = PERM ? (int)__reduce_min_sync(FULL, me ? (unsigned)cx : 0xffffffffu)
				     : __shfl_sync(FULL, pcx, __ffs(pm) - 1);
		const int xhi = PERM ? (int)__reduce_max_sync(FULL, me ? (unsigned)cx : 0u)
				     : __shfl_sync(FULL, pcx, 31 - __clz(pm));
		const int ry = rrow % nc1, rz = rrow / nc1;
		// the staged region spans (xhi - xlo + 3) x 3 x 3 cells; when that is
		// under half the box on every axis, separations need no wrapping
		local = 2 * (xhi - xlo + 3) < nc0 && 6 < nc1 && 6 < nc2;
		// the frame: the run's first particle
		const int rl0 = TB == 2 ? __ffs(pm) - 1 : leader;
		ref.x = __shfl_sync(FULL, ppi.x, rl0);
		ref.y = __shfl_sync(FULL, ppi.y, rl0);
		ref.z = __shfl_sync(FULL, ppi.z, rl0);
		mx = sep_hi(pi.x, ref.x, a.fs[0]);
		my = sep_hi(pi.y, ref.y, a.fs[1]);
		mz = sep_hi(pi.z, ref.z, a.fs[2]);
		// bounding box of the run's particles, widened by rlist at use
		bx0 = warp_min_f(me ? mx : 3.0e38f, FULL); bx1 = warp_max_f(me ? mx : -3.0e38f, FULL);
		by0 = warp_min_f(me ? my : 3.0e38f, FULL); by1 = warp_max_f(me ? my : -3.0e38f, FULL);
		bz0 = warp_min_f(me ? mz : 3.0e38f, FULL); bz1 = warp_max_f(me ? mz : -3.0e38f, FULL);
		// A wrapped region (small boxes) drops candidates whose periodic
		// distance from the run's bounding box is rlist or more: per axis
		// the gap between the candidate's offset and the box's interval,
		// over the nearest image (offsets and the interval lie within half
		// a box of the run's first particle, so |o - centre| < L and the
		// nearer image is at L - |o - centre|).  Every member's minimum-image
		// separation is at least that distance on each axis.  rlm carries a
		// margin for the roundings, so the filter only removes candidates
		// the test would reject, and the list is the same with or without it.
		const float cxm = 0.5f * (bx0 + bx1), hxm = 0.5f * (bx1 - bx0);
		const float cym = 0.5f * (by0 + by1), hym = 0.5f * (by1 - by0);
		const float czm = 0.5f * (bz0 + bz1), hzm = 0.5f * (bz1 - bz0);
		const float Lx = a.fs[0] * 4294967296.f, Ly = a.fs[1] * 4294967296.f, Lz = a.fs[2] * 4294967296.f;
		int sA0, sA1, sB0 = 0, sB1 = 0;
		if (xhi - xlo + 3 >= nc0) { sA0 = 0; sA1 = nc0; }
		else {
			const int s0 = xlo - 1, s1 = xhi + 2;
			if (s0 < 0) { sA0 = s0 + nc0; sA1 = nc0; sB1 = s1; }
			else if (s1 > nc0) { sA0 = s0; sA1 = nc0; sB1 = s1 - nc0; }
			else { sA0 = s0; sA1 = s1; }
		}
		// the run's candidate segments, in staging order: up to 9 rows x 2
		// x-ranges; lane k loads segment k's bounds, all in one round
		int nseg = 0, seg_b = 0, seg_e = 0;
		for (int oz = lo2; oz <= hi2; oz++) {
			const int zz = wrapc(rz + oz, nc2);
			for (int oy = lo1; oy <= hi1; oy++) {
				const int yy = wrapc(ry + oy, nc1);
				const int rb = nc0 * (yy + nc1 * zz);
				for (int sg = 0; sg < 2; sg++) {
					const int c0 = sg ? sB0 : sA0, c1 = sg ? sB1 : sA1;
					if (c1 <= c0) continue;
					if (lane == nseg) { seg_b = a.cellstart[rb + c0]; seg_e = a.cellstart[rb + c1]; }
					nseg++;
				}
			}
		}
		// chunks of up to 32 consecutive candidates; the loads of the next
		// chunk are issued before the current one is filtered and tested
		int sidx = 0, jj = 0, je = 0;
		auto next_seg = [&]() {
			while (sidx < nseg) {
				jj = __shfl_sync(FULL, seg_b, sidx);
				je = __shfl_sync(FULL, seg_e, sidx);
				if (jj < je) return;
				sidx++;
			}
		};
		next_seg();
		int4 pn = make_int4(0, 0, 0, 0);
		int mn = 0, jn = 0;
		if (sidx < nseg && lane < je - jj) {
			jn = PERM ? a.perm[jj + lane] : jj + lane;
			pn = a.pos[jn];
			if (MOLX) mn = a.mol[jn];
		}
		int fill = 0;
		while (sidx < nseg) {
			const int take = min(32, je - jj);
			const int4 pj = pn;
			const int mj = mn, jcur = jn;
			jj += 32;
			if (jj >= je) { sidx++; next_seg(); }
			if (sidx < nseg && lane < min(32, je - jj)) {
				jn = PERM ? a.perm[jj + lane] : jj + lane;
				pn = a.pos[jn];
				if (MOLX) mn = a.mol[jn];
			}
			if (fill + take > BT_CAP) { test(fill); fill = 0; }
			bool keep = lane < take;
			float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
			if (keep) {
				if (local) {
					q = make_float4(sep_hi(pj.x, ref.x, a.fs[0]), sep_hi(pj.y, ref.y, a.fs[1]),
							sep_hi(pj.z, ref.z, a.fs[2]), __int_as_float(jcur));
					const float ex = fmaxf(fmaxf(bx0 - q.x, q.x - bx1), 0.f);
					const float ey = fmaxf(fmaxf(by0 - q.y, q.y - by1), 0.f);
					const float ez = fmaxf(fmaxf(bz0 - q.z, q.z - bz1), 0.f);
					keep = ex < rl && ey < rl && ez < rl && fmaf(ex, ex, fmaf(ey, ey, ez * ez)) < a.rl2;
				} else {
					q = make_float4(__int_as_float(pj.x), __int_as_float(pj.y), __int_as_float(pj.z),
							__int_as_float(jcur));
					const float dx = fabsf(sep_hi(pj.x, ref.x, a.fs[0]) - cxm);
					const float dy = fabsf(sep_hi(pj.y, ref.y, a.fs[1]) - cym);
					const float dz = fabsf(sep_hi(pj.z, ref.z, a.fs[2]) - czm);
					const float ex = fmaxf(fminf(dx, Lx - dx) - hxm, 0.f);
					const float ey = fmaxf(fminf(dy, Ly - dy) - hym, 0.f);
					const float ez = fmaxf(fminf(dz, Lz - dz) - hzm, 0.f);
					keep = ex < rlm && ey < rlm && ez < rlm &&
					       fmaf(ex, ex, fmaf(ey, ey, ez * ez)) < rlm * rlm;
				}
			}
			const unsigned kb = __ballot_sync(FULL, keep);
			if (keep) {
				const int slot = fill + __popc(kb & ((1u << lane) - 1u));
				sp[slot] = q;
				if (MOLX) spm[slot] = mj;
			}
			fill += __popc(kb);
		}
		test(fill);
	}
	__syncwarp();
	flush();
	if (own) {
		a.ncnt[i] = cnt < cap ? cnt : cap;
		if (cnt > cap) atomicOr(&a.flags[0], 1u);
	}
	const unsigned mxc = __reduce_max_sync(FULL, own ? (unsigned)cnt : 0u);
	if (lane == 0) atomicMax(&a.flags[1], mxc);
}

template <int TB>
__global__ void __launch_bounds__(BT_WARPS * 32) k_build_tiles(long n, BuildArgs a)
{
	__shared__ float4 sp_all[BT_WARPS][BT_CAP];
	__shared__ int ring_all[BT_WARPS][BT_RING * 32];
	const int w = threadIdx.x >> 5;
	build_tile<false, false, false, TB>(n, a, ((long)blockIdx.x * BT_WARPS + w) * (32 / TB), sp_all[w],
					    ring_all[w]);
}

// Same-molecule exclusions (the butane-type workloads): molecule indices
// staged with the candidates.
template <int TB>
__global__ void __launch_bounds__(BT_WARPS * 32) k_build_tiles_mol(long n, BuildArgs a)
{
	__shared__ float4 sp_all[BT_WARPS][BT_CAP];
	__shared__ int spm_all[BT_WARPS][BT_CAP];
	__shared__ int ring_all[BT_WARPS][BT_RING * 32];
	const int w = threadIdx.x >> 5;
	build_tile<false, true, false, TB>(n, a, ((long)blockIdx.x * BT_WARPS + w) * (32 / TB), sp_all[w],
					   ring_all[w], spm_all[w]);
}

// Batched systems: each warp builds its tile with its own system's cell grid
// and box, and only for systems whose rebuild flag is set.
// fw (with its count fcnt) lists the flagged systems' warps: a fixed grid
// steps through it; without it, a warp per 32 slots of every system, the
// unflagged ones leaving at once
__global__ void __launch_bounds__(BT_WARPS * 32) k_build_tiles_batch(BuildArgs a, const BatchSys *sys,
								    const int *wsys, int nwarps,
								    const unsigned *flag, const int *fw,
								    const int *fcnt)
{
	__shared__ float4 sp_all[BT_WARPS][BT_CAP];
	__shared__ int ring_all[BT_WARPS][BT_RING * 32];
	const int w = threadIdx.x >> 5;
	auto tile = [&](long wg) {
		const BatchSys S = sys[wsys[wg]];
		BuildArgs b = a;
		b.cellstart = a.cellstart + S.coff;
		for (int k = 0; k < 3; k++) { b.nc[k] = S.nc[k]; b.fs[k] = S.fs; }
		build_tile<true>(S.off + S.n, b, wg * 32, sp_all[w], ring_all[w]);
	};
	if (fw) {
		for (long k = (long)blockIdx.x * BT_WARPS + w; k < *fcnt; k += (long)gridDim.x * BT_WARPS) tile(fw[k]);
	} else {
		const long wg = (long)blockIdx.x * BT_WARPS + w;
		if (wg >= nwarps || !flag[wsys[wg]]) return;
		tile(wg);
	}
}

// The same over index-only cell lists (particles not moved: the adjoint).
__global__ void __launch_bounds__(BT_WARPS * 32) k_build_tiles_batch_perm(BuildArgs a, const BatchSys *sys,
									 const int *wsys, int nwarps,
									 const unsigned *flag)
{
	__shared__ float4 sp_all[BT_WARPS][BT_CAP];
	__shared__ int ring_all[BT_WARPS][BT_RING * 32];
	const int w = threadIdx.x >> 5;
	const long wg = (long)blockIdx.x * BT_WARPS + w;
	if (wg >= nwarps) return;
	const int s = wsys[wg];
	if (!flag[s]) return;
	const BatchSys S = sys[s];
	BuildArgs b = a;
	b.cellstart = a.cellstart + S.coff;
	for (int k = 0; k < 3; k++) { b.nc[k] = S.nc[k]; b.fs[k] = S.fs; }
	build_tile<true, false, true>(S.off + S.n, b, wg * 32, sp_all[w], ring_all[w]);
}

// Deterministic order inside each cell: one warp per cell ranks its members
// by x, ties by user index (dev_cellsort.cuh).  Launched with 256 threads.
__global__ void __launch_bounds__(256) k_cellsort_w(long m, const int *__restrict__ start,
						    const int *__restrict__ gid, const int4 *__restrict__ pos,
						    int *__restrict__ perm)
{
	__shared__ unsigned long long sk[8][CS_MAX];
	__shared__ int sv[8][CS_MAX];
	const long c = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
	if (c >= m) return;
	const int w = threadIdx.x >> 5;
	const int lo = start[c];
	cell_sort_warp(lo, start[c + 1] - lo, gid, pos, perm, sk[w], sv[w]);
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
	const float4 *ext_s[SEPDEV_NEXT]; float4 *ext_d[SEPDEV_NEXT];
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
#pragma unroll
	for (int k = 0; k < SEPDEV_NEXT; k++)
		if (a.ext_s[k]) a.ext_d[k][t] = a.ext_s[k][t];
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

// the system's team size (lanes per particle) also sets the build's lanes
// per particle; the lists are the same either way
static int launch_build(sepdev *d, const BuildArgs &a)
{
	const int tb = d->team == 2 ? 2 : 1, per = 32 / tb;
	const int grid = grid_for((d->n + per - 1) / per, BT_WARPS);
	if (a.excl == SEPDEV_EXCL_SAMEMOL) {
		if (tb == 2) k_build_tiles_mol<2><<<grid, BT_WARPS * 32, 0, d->st>>>(d->n, a);
		else k_build_tiles_mol<1><<<grid, BT_WARPS * 32, 0, d->st>>>(d->n, a);
	} else {
		if (tb == 2) k_build_tiles<2><<<grid, BT_WARPS * 32, 0, d->st>>>(d->n, a);
		else k_build_tiles<1><<<grid, BT_WARPS * 32, 0, d->st>>>(d->n, a);
	}
	CKL(d);
	return SEPDEV_OK;
}

// Cell grid for cut-off rlist: edge >= cellf * rlist (cellf >= 1, from the
// tuning table), total cells bounded by 2n + 64.
static int cell_grid(sepdev *d, double rlist)
{
	for (int k = 0; k < 3; k++) {
		int c = (int)floor(d->L[k] / (rlist * d->cellf));
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
	k_cellsort_w<<<grid_for(d->ncells * 32, B), B, 0, d->st>>>(d->ncells, d->cellstart, d->gid, d->pos[parity],
								  d->perm);
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
	for (int k = 0; k < SEPDEV_NEXT; k++) { g.ext[k] = d->ext[k]; g.ext_o[k] = d->ext_b[k]; }
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
	for (int k = 0; k < SEPDEV_NEXT; k++) { c.ext_s[k] = d->ext_b[k]; c.ext_d[k] = d->ext[k]; }
	k_copyback<<<grid_for(n, B), B, 0, d->st>>>(n, c);
	CKL(d);
	return SEPDEV_OK;
}

static int list_capacity(sepdev *d, int maxnb)
{
	maxnb = ((maxnb + 7) / 8) * 8;
	const size_t tiles = (size_t)((d->n + 31) / 32);
	const size_t bytes = tiles * 32 * (size_t)maxnb * sizeof(int);
	int rc = grow(d, (void **)&d->nl, bytes, &d->cap_nl);
	if (rc) return rc;
	d->maxnb = maxnb;
	return SEPDEV_OK;
}

// capacity for at least maxnb neighbours per particle (existing lists are lost)
int sepdev_grow_list_to(sepdev *d, int maxnb)
{
	return list_capacity(d, maxnb);
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
	a->perm = NULL;
	return SEPDEV_OK;
}

int sepdev_batch_build(sepdev *d, int parity, const int *cellstart, const BatchSys *sys,
		       const int *wsys, int nwarps, const unsigned *flag, float rl2, const int *perm,
		       const int *fw, const int *fcnt)
{
	BuildArgs a;
	memset(&a, 0, sizeof a);
	a.pos = d->pos[parity];
	a.cellstart = cellstart;
	a.rl2 = rl2;
	a.maxnb = d->maxnb;
	a.nl = d->nl;
	a.ncnt = d->ncnt;
	a.flags = d->flags;
	a.excl = SEPDEV_EXCL_NONE;
	a.gid = d->gid;
	a.mol = d->mol;
	a.perm = perm;
	if (perm)
		k_build_tiles_batch_perm<<<grid_for(nwarps, BT_WARPS), BT_WARPS * 32, 0, d->st>>>(a, sys, wsys, nwarps,
												   flag);
	else if (fw)
		k_build_tiles_batch<<<6 * d->nsm, BT_WARPS * 32, 0, d->st>>>(a, sys, wsys, nwarps, flag, fw, fcnt);
	else
		k_build_tiles_batch<<<grid_for(nwarps, BT_WARPS), BT_WARPS * 32, 0, d->st>>>(a, sys, wsys, nwarps, flag,
											     NULL, NULL);
	CKL(d);
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

// The host-driven rebuild's first part: kernel parameters, cell grid, sort
// (asynchronous), and a first list capacity from the mean density.
static int list_prepare(sepdev *d, double rlist, int excl, int trigger)
{
	if (!(rlist > 0)) return SEPDEV_EINVAL;
	if ((excl == SEPDEV_EXCL_BONDS || excl == SEPDEV_EXCL_ALLBONDED) && !d->has_excl)
		excl = SEPDEV_EXCL_NONE;
	d->rlist = rlist;
	d->excl = excl;
	// the kernel parameters of the system's size class, as tuned
	sepdev_tuning_for(d->n, &d->team, &d->groups, &d->cellf);
	int rc;
	if ((rc = cell_grid(d, rlist))) return rc;
	if ((rc = sepdev_sort_async(d, d->cur, trigger))) return rc;
	if (d->maxnb == 0) {
		const double vol = d->L[0] * d->L[1] * d->L[2];
		const double est = 4.18879020479 * rlist * rlist * rlist * (double)d->n / vol;
		if ((rc = list_capacity(d, (int)(1.35 * est) + 32))) return rc;
	}
	return SEPDEV_OK;
}

// Build from the sorted order, check the capacity, grow it and build again
// when a particle overflowed (synchronous).
static int build_checked(sepdev *d)
{
	int rc;
	for (int attempt = 0; attempt < 4; attempt++) {
		if ((rc = sepdev_build_async(d, d->cur))) return rc;
		unsigned fl[2];
		CK(cudaMemcpyAsync(fl, d->flags, sizeof fl, cudaMemcpyDeviceToHost, d->st));
		CK(cudaStreamSynchronize(d->st));
		if (!(fl[0] & 1u)) {
			d->list_valid = 1;
			d->list_unchecked = 0;
			return SEPDEV_OK;
		}
		if ((rc = list_capacity(d, (int)(fl[1] * 1.25) + 16))) return rc;
	}
	return SEPDEV_EOVERFLOW;
}

// Host-driven rebuild: sort, build, check the capacity and grow it when a
// particle overflowed (synchronous).
extern "C" int sepdev_build_list(sepdev *d, double rlist, int excl, int trigger)
{
	int rc;
	if ((rc = list_prepare(d, rlist, excl, trigger))) return rc;
	return build_checked(d);
}

// The same without waiting: the list is marked unchecked.  A step kernel
// skips its work when the build overflowed (flags[0]); the next read of
// the flags with the step's sums (sepdev_slots_take) clears the mark, and
// every other consumer confirms the list first (sepdev_list_confirm).
extern "C" int sepdev_build_list_deferred(sepdev *d, double rlist, int excl, int trigger)
{
	int rc;
	if ((rc = list_prepare(d, rlist, excl, trigger))) return rc;
	if ((rc = sepdev_build_async(d, d->cur))) return rc;
	d->list_valid = 1;
	d->list_unchecked = 1;
	return SEPDEV_OK;
}

// Settle an unchecked list: read the overflow flag, and on overflow grow the
// capacity and build again from the same sorted order (synchronous).
extern "C" int sepdev_list_confirm(sepdev *d)
{
	if (!d->list_unchecked) return SEPDEV_OK;
	unsigned fl[2];
	CK(cudaMemcpyAsync(fl, d->flags, sizeof fl, cudaMemcpyDeviceToHost, d->st));
	CK(cudaStreamSynchronize(d->st));
	if (!(fl[0] & 1u)) {
		d->list_unchecked = 0;
		return SEPDEV_OK;
	}
	int rc;
	if ((rc = list_capacity(d, (int)(fl[1] * 1.25) + 16))) return rc;
	return build_checked(d);
}

// Grow the list for a count the device reported (used after an in-graph overflow).
int sepdev_grow_list(sepdev *d, int needed)
{
	return list_capacity(d, (int)(needed * 1.25) + 16);
}

extern "C" int sepdev_list_stats(sepdev *d, int *maxcount, double *meancount, int *capacity)
{
	if (!d->list_valid || !d->ncnt) return SEPDEV_EINVAL;
	int rc;
	if ((rc = sepdev_list_confirm(d))) return rc;
	int *h = (int *)malloc(sizeof(int) * d->n);
	if (!h) return SEPDEV_ENOMEM;
	cudaError_t e = cudaMemcpyAsync(h, d->ncnt, sizeof(int) * d->n, cudaMemcpyDeviceToHost, d->st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
	if (e != cudaSuccess) { free(h); sepdev_set_error("list stats", e); return SEPDEV_ECUDA; }
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
	if (!d->list_valid || sepdev_list_confirm(d)) return -1;
	const long n = d->n;
	const size_t len = (size_t)((n + 31) / 32) * 32 * (size_t)d->maxnb;
	int *nl = (int *)malloc(sizeof(int) * len), *cnt = (int *)malloc(sizeof(int) * n);
	int *gid = (int *)malloc(sizeof(int) * n);
	if (!nl || !cnt || !gid) { free(nl); free(cnt); free(gid); return -2; }
	cudaMemcpyAsync(nl, d->nl, sizeof(int) * len, cudaMemcpyDeviceToHost, d->st);
	cudaMemcpyAsync(cnt, d->ncnt, sizeof(int) * n, cudaMemcpyDeviceToHost, d->st);
	cudaMemcpyAsync(gid, d->gid, sizeof(int) * n, cudaMemcpyDeviceToHost, d->st);
	if (cudaStreamSynchronize(d->st) != cudaSuccess) { free(nl); free(cnt); free(gid); return -3; }
	long np = 0;
	for (long i = 0; i < n; i++) {
		for (int k = 0; k < cnt[i]; k++) {
			const int j = nl[nl_index(i, k, d->maxnb)];
			const int gi = gid[i], gj = gid[j];
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

extern "C" void sepdev_params(sepdev *d, int *team, int *groups, double *cellf)
{
	if (team) *team = d->team;
	if (groups) *groups = d->groups;
	if (cellf) *cellf = d->cellf;
}
