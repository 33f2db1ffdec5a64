// dev_common.cuh - internals shared by the sepdev translation units.
//
// Number formats (chosen for GB300, whose FP64 rate is 1/64 of FP32):
//  * position component k: unsigned 64-bit fixed point X = frac * 2^64 with
//    frac = x / L_k in [0, 1).  The high word (x_hi) is what the pair kernels
//    read; (int)(x_hi_i - x_hi_j) is the minimum-image separation in units of
//    L_k / 2^32 because two's-complement wrap-around is the periodic boundary.
//    The integrator adds v dt in this format, so the position update keeps
//    more than FP64 resolution (L / 2^64) without a single FP64 instruction.
//  * velocity: float-float (hi + lo, ~48-bit mantissa).
//  * per-pair force, energy and virial: FP32.
//  * sums over particles: every particle's term is converted exactly to 64-bit
//    fixed point (scale 2^32) and summed with integer warp reductions and
//    integer atomics, so every total is exact to 2^-32 per term and
//    independent of scheduling order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include "../sepdev.h"

#define SEPDEV_NEV 8
#define SEPDEV_MAXTAB 4

struct sepdev {
	long n;
	int device;
	cudaStream_t st;
	cudaEvent_t ev[SEPDEV_NEV];

	double L[3];
	float fscale[3];        // L_k / 2^32
	double vscale_hi[3], vscale_lo[3];  // unused placeholder for alignment

	// particle state in cell order
	int4 *pos[2];           // x_hi, y_hi, z_hi, type id
	int cur;
	uint4 *xlo, *xlo_b;     // low words, .w = 0
	float4 *vhi, *vhi_b;    // velocity hi, .w = mass
	float4 *vlo, *vlo_b;    // velocity lo, .w = 1/mass
	float4 *frc, *frc_b;    // force, .w = per-particle pair energy
	int4 *xn;               // high words at the last list build
	int4 *cross, *cross_b;  // crossings since the start
	int4 *cbase, *cbase_b;  // crossings at the last skin-triggered build
	int *gid, *gid_b;       // user index of each slot
	int *inv;               // slot of each user index
	float *charge, *charge_b;
	int *mol, *mol_b;
	int has_charge;

	// stochastic-dynamics fields, allocated on first use (NULL otherwise):
	// [SEPDEV_EXT_PV] predicted velocity, .w = Langevin diffusion
	// coefficient; [SEPDEV_EXT_PA] previous acceleration; [SEPDEV_EXT_PREVF]
	// previous force; [SEPDEV_EXT_RANDN] the last Gaussian draws (GJF)
	float4 *ext[SEPDEV_NEXT], *ext_b[SEPDEV_NEXT];

	// molecular pressure tensor (sepdev_molvir_enable): molecule tables in
	// user indices, centres of mass of the last pair pass and its box, the
	// per-atom intermolecular force since the last reset (user order)
	// per-type operations (dev_typeops.cu): tether positions x0 (user
	// order, 3 doubles each), scratch for sums and profile histograms
	double *x0;
	void *tscr;
	size_t tscr_cap;

	int molvir_on, nmolv;
	int *mv_first, *mv_nuau, *mv_start, *mv_atoms;
	double *mv_mass;
	int4 *mv_cm;
	float4 *mv_finter;
	double *mv_out;
	double mv_L[3];
	int mv_slot;            // slot the next pair pass writes its molecular sums to

	// cell list
	int ncell[3];
	long ncells, cap_cells;
	int *cellof;            // cell of each slot (old order)
	int *celloff;           // rank inside the cell
	int *cellcount;
	int *cellstart;         // ncells + 1
	int *perm;              // new slot -> old slot

	// neighbour list: tiles of 32 particles, each tile maxnb * 32 ints (nl_index)
	int *nl;
	int *ncnt;
	int maxnb;
	// kernel parameters of the system's size class (the tuning table),
	// taken at every list build: lanes per particle, neighbour groups per
	// iteration, cell edge over the list cut-off
	int team, groups;
	double cellf;
	size_t cap_nl;
	double rlist;
	int excl;
	int list_valid;
	int list_unchecked;       // built without the capacity check: the next read of the flags decides

	// exclusions (user indices, CSR)
	int *exb_start, *exb_idx, *exa_start, *exa_idx;
	int has_excl;

	// topology (user indices) and per-atom incidence CSR
	int nbond, nangle, ndihed;
	uint4 *bonds;           // a b type -
	uint4 *angles;          // a b c type
	uint4 *diheds_abcd;     // a b c d
	int *dihed_type;
	int *inc_start;         // n+1, per user atom
	int *inc_term;          // encoded term: kind<<30 | role<<28 | index
	float *term_out;        // per-term observable (length / angle)
	size_t term_out_cap;

	// tabulated potentials
	float2 *tab[SEPDEV_MAXTAB];
	int tab_n[SEPDEV_MAXTAB];
	float tab_r2min[SEPDEV_MAXTAB], tab_idr2[SEPDEV_MAXTAB];

	// reductions
	long long *slots;       // device, nslots * SLOT_FIELDS
	long long *h_slots;     // pinned, mapped mirror (host address)
	long long *hd_slots;    // the same memory, device address
	unsigned *flags;        // device status word [0] overflow, [1] max count, [2..3] scratch
	unsigned *h_flags;      // pinned, mapped mirror (host address)
	unsigned *hd_flags;     // the same memory, device address
	unsigned *take_arrive;  // device: arrival count of a step kernel that hands its sums over
	int take_ready;         // slots a step kernel handed over for the next read (-1: none)
	int nslots;

	sepdev_pairset *d_ps;   // device copy of the current pair set
	sepdev_pairset h_ps;    // what d_ps holds (uploads are skipped when unchanged)
	int ps_valid;

	// graph runner state
	void *runner;

	// L2 flush buffer of the timing helpers (allocated on first use)
	void *flush_buf;
	size_t flush_bytes;

	// pinned host staging of uploads and downloads (kept between calls)
	void *stage;
	size_t stage_bytes;

	// in-place transfers: the device reads and writes the seppart array
	// itself (set when the GPU can address pageable host memory)
	int hostio_direct;
	void *hio_scr;
	size_t hio_bytes;

	int nsm;                // streaming multiprocessors of the device

	long launches;
};

#define FX_SCALE 4294967296.0f      // 2^32
#define FX_ISCALE (1.0 / 4294967296.0)

// ---- error handling -------------------------------------------------------
extern "C" void sepdev_set_error(const char *what, cudaError_t e);
#define CK(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) { \
	sepdev_set_error(#call, e_); return SEPDEV_ECUDA; } } while (0)
#define CKL(d) do { (d)->launches++; cudaError_t e_ = cudaGetLastError(); \
	if (e_ != cudaSuccess) { sepdev_set_error("kernel launch", e_); return SEPDEV_ECUDA; } } while (0)

// ---- small device helpers -------------------------------------------------
// reciprocal: hardware approximation refined by one Newton step, which
// removes the approximation's bias (the result is within ~0.5 ulp)
__device__ __forceinline__ float fast_rcp(float x)
{
	float r;
	asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
	const float e = fmaf(-x, r, 1.0f);
	return fmaf(r, e, r);
}

// minimum-image separation component from two high words
__device__ __forceinline__ float sep_hi(int a, int b, float s)
{
	return (float)(a - b) * s;
}

// float-float: (hi, lo) + q, returns renormalised pair
__device__ __forceinline__ void ff_add(float &hi, float &lo, float q)
{
	const float s = __fadd_rn(hi, q);
	const float bp = __fsub_rn(s, hi);
	float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(q, bp));   // two-sum error
	e = __fadd_rn(e, lo);
	const float h2 = __fadd_rn(s, e);
	lo = __fsub_rn(e, __fsub_rn(h2, s));
	hi = h2;
}

// 64-bit fixed-point increment round((hi + lo) * (shi + slo)) with
// |result| < 2^62; exact product of the high parts via FMA
// (explicit roundings throughout, so every kernel that inlines it computes
// the same bits whatever the compiler contracts around it)
__device__ __forceinline__ long long ff_mul_fix(float hi, float lo, float shi, float slo)
{
	const float p = __fmul_rn(hi, shi);
	const float e = __fmaf_rn(hi, shi, -p);
	const float r = __fadd_rn(e, __fmaf_rn(hi, slo, __fmul_rn(lo, shi)));
	return __float2ll_rn(p) + __float2ll_rn(r);
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31; }

// Fixed-point value (units of 2^-32, rounded to the nearest unit) of a
// float.  The 64-bit float-to-integer conversion runs at a small fraction of
// the 32-bit rates, so for |v| < 2^22 the value is split exactly: n =
// round(v) by the 1.5 * 2^23 addition (full-rate FP32), f = v - n exactly
// (|f| <= 1/2, Sterbenz), and f * 2^32 converted with one 32-bit conversion.
// Larger values (or NaN) take the 64-bit conversion.
__device__ __forceinline__ long long to_fx(float v)
{
	if (!(fabsf(v) < 4194304.0f)) return __float2ll_rn(v * FX_SCALE);
	const float M = 12582912.0f;
	const float t = __fadd_rn(v, M);
	const int n = __float_as_int(t) - 0x4B400000;
	const float f = __fsub_rn(v, __fsub_rn(t, M));
	// |f 2^32| <= 2^31: the one value that does not fit (f = 1/2) saturates,
	// an error of one unit
	const int lo = __float2int_rn(__fmul_rn(f, FX_SCALE));
	return (long long)n * 4294967296ll + (long long)lo;
}

// the same for a float-float (h + l, |l| <= ulp(h)/2, |h| < 2^23)
__device__ __forceinline__ long long to_fx2(float h, float l)
{
	return to_fx(h) + (long long)__float2int_rn(__fmul_rn(l, FX_SCALE));
}

// m * a * b for float-float a and b, as a float-float (hi, lo): the product
// of the high parts is split exactly with an FMA; the cross terms and the
// mass factor carry the rest (relative error ~2^-44).  Every product and
// sum is an explicit rounding, so no compiler contraction changes the bits.
__device__ __forceinline__ void ff_mprod(float m, float ah, float al, float bh, float bl, float &hi,
					 float &lo)
{
	const float p = __fmul_rn(ah, bh);
	const float e = __fadd_rn(__fmaf_rn(ah, bh, -p), __fmaf_rn(ah, bl, __fmul_rn(al, bh)));
	hi = __fmul_rn(m, p);
	lo = __fadd_rn(__fmaf_rn(m, p, -hi), __fmul_rn(m, e));
}

// Exact warp sum of 64-bit fixed-point values (result in every lane): the
// high words and the two 16-bit halves of the low words are summed
// separately with integer warp reductions, so no carry is lost.  The high
// words' sum must fit in 32 bits (|sum| < 2^31 units of 1).
__device__ __forceinline__ long long warp_sum_fx(long long q)
{
	const unsigned FULL = 0xffffffffu;
	const unsigned lo = (unsigned)q;
	const int shi = __reduce_add_sync(FULL, (int)(q >> 32));
	const unsigned smid = __reduce_add_sync(FULL, lo >> 16);
	const unsigned slo = __reduce_add_sync(FULL, lo & 0xffffu);
	return ((long long)shi << 32) + ((long long)smid << 16) + (long long)slo;
}

// Block reduction of NV fixed-point values: base[fld[k]] += sum q[k] through
// 64-bit integer atomics, exact at every level (so totals do not depend on
// the order of anything), plus an optional max of a non-negative float into
// base[maxfld] (maxfld < 0: none).  Must be called by all threads of the
// block, once per kernel.
template <int NV>
__device__ __forceinline__ void block_to_slot_fx(const long long (&q)[NV], const int (&fld)[NV],
						 long long *base, float maxval, int maxfld)
{
	__shared__ long long red[32][NV];
	__shared__ unsigned redm[32];
	const unsigned mx = __reduce_max_sync(0xffffffffu, __float_as_uint(maxval));
	const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
	for (int k = 0; k < NV; k++) {
		const long long s = warp_sum_fx(q[k]);
		if (lane_id() == 0) red[w][k] = s;
	}
	if (lane_id() == 0) redm[w] = mx;
	__syncthreads();
	if (w == 0) {
#pragma unroll
		for (int k = 0; k < NV; k++) {
			const long long s = warp_sum_fx((int)lane_id() < nw ? red[lane_id()][k] : 0ll);
			if (lane_id() == 0 && s != 0)
				atomicAdd((unsigned long long *)&base[fld[k]], (unsigned long long)s);
		}
		if (maxfld >= 0) {
			unsigned m = (int)lane_id() < nw ? redm[lane_id()] : 0u;
			m = __reduce_max_sync(0xffffffffu, m);
			if (lane_id() == 0 && m)
				atomicMax((unsigned long long *)&base[maxfld], (unsigned long long)m);
		}
	}
}

// Block reduction of NV per-thread floats (each converted exactly to fixed
// point first), as block_to_slot_fx.
template <int NV>
__device__ __forceinline__ void block_to_slot(const float (&v)[NV], const int (&fld)[NV],
					      long long *base, float maxval, int maxfld)
{
	long long q[NV];
#pragma unroll
	for (int k = 0; k < NV; k++) q[k] = to_fx(v[k]);
	block_to_slot_fx<NV>(q, fld, base, maxval, maxfld);
}

// host to_fixed (dev_state.cu) with the same operations and roundings
__device__ __forceinline__ void to_fixed_dev(double x, double L, unsigned &hi, unsigned &lo)
{
	double fr = __ddiv_rn(x, L);
	fr = __dsub_rn(fr, floor(fr));
	if (fr >= 1.0) fr = 0.0;
	const double t = ldexp(fr, 32);
	const double h = floor(t);
	const double r = ldexp(__dsub_rn(t, h), 32);
	hi = (unsigned)h;
	lo = (unsigned)floor(r);
}

__device__ __forceinline__ double from_fixed_dev(unsigned hi, unsigned lo, double L)
{
	return __dmul_rn(__dadd_rn(ldexp((double)hi, -32), ldexp((double)lo, -64)), L);
}

// Neighbour-list layout (one lane per particle): particle i is lane
// p = i % 32 of tile t = i / 32; its entry k lives at
//     nl[t*maxnb*32 + (k/4)*128 + p*4 + (k%4)]
// so a lane's next four neighbours are one 16-byte load and a warp's batch
// of four is one contiguous 512-byte read.  maxnb is a multiple of 8.
__host__ __device__ __forceinline__ long nl_index(long i, int k, int maxnb)
{
	return (i >> 5) * (long)maxnb * 32 + (long)(k >> 2) * 128 + (i & 31) * 4 + (k & 3);
}

static inline int grid_for(long n, int block) { return (int)((n + block - 1) / block); }
