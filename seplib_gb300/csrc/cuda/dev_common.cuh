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
//  * sums over particles: FP32 within a warp (<= 32 particles), then exact
//    64-bit fixed point (scale 2^32) through integer atomics, so every total is
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

	// neighbour list: tiles of 32/tpp particles, each tile maxnb*(32/tpp) ints
	int *nl;
	int *ncnt;
	int maxnb, tpp;
	size_t cap_nl;
	double rlist;
	int excl;
	int list_valid;

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
	long long *h_slots;     // pinned mirror
	unsigned *flags;        // device status word [0] overflow, [1] max count, [2..3] scratch
	unsigned *h_flags;      // pinned mirror
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

	// kernel variants chosen by the tuner (SEPLIB_LJ_VARIANT overrides)
	int lj_variant;
	int nsm;

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
	float s = hi + q;
	float bp = s - hi;
	float e = (hi - (s - bp)) + (q - bp);   // two-sum error
	e += lo;
	float h2 = s + e;
	lo = e - (h2 - s);
	hi = h2;
}

// 64-bit fixed-point increment round((hi + lo) * (shi + slo)) with
// |result| < 2^62; exact product of the high parts via FMA
__device__ __forceinline__ long long ff_mul_fix(float hi, float lo, float shi, float slo)
{
	float p = hi * shi;
	float e = fmaf(hi, shi, -p);
	float r = e + (hi * slo + lo * shi);
	return __float2ll_rn(p) + __float2ll_rn(r);
}

// ---- packed FP32 pairs (f32x2 instructions of sm_100-family GPUs) --------
// Two floats in one 64-bit register; one instruction operates on both.
typedef unsigned long long f2_t;
__device__ __forceinline__ f2_t f2_pack(float a, float b)
{
	f2_t r;
	asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
	return r;
}
__device__ __forceinline__ void f2_unpack(f2_t r, float &a, float &b)
{
	asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ f2_t f2_fma(f2_t a, f2_t b, f2_t c)
{
	f2_t d;
	asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
	return d;
}
__device__ __forceinline__ f2_t f2_mul(f2_t a, f2_t b)
{
	f2_t d;
	asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
	return d;
}
__device__ __forceinline__ f2_t f2_add(f2_t a, f2_t b)
{
	f2_t d;
	asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
	return d;
}
__device__ __forceinline__ f2_t f2_sub(f2_t a, f2_t b)
{
	f2_t d;
	asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
	return d;
}
__device__ __forceinline__ float f2_sum(f2_t r)
{
	float a, b;
	f2_unpack(r, a, b);
	return a + b;
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31; }

// Warp sum of NV floats, result valid in lane 0.
template <int NV>
__device__ __forceinline__ void warp_sum(float (&v)[NV])
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1)
#pragma unroll
		for (int k = 0; k < NV; k++) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
}

// Block reduction of NV floats: base[fld[k]] += sum v[k] through 64-bit
// fixed-point atomics (FP32 inside each warp, exact integer sums above), plus
// an optional max of a non-negative float into base[maxfld] (maxfld < 0: none).
// Must be called by all threads of the block, once per kernel.
template <int NV>
__device__ __forceinline__ void block_to_slot(float (&v)[NV], const int (&fld)[NV],
					      long long *base, float maxval, int maxfld)
{
	__shared__ long long red[32][NV];
	__shared__ unsigned redm[32];
	warp_sum<NV>(v);
	const unsigned mx = __reduce_max_sync(0xffffffffu, __float_as_uint(maxval));
	const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
	if (lane_id() == 0) {
#pragma unroll
		for (int k = 0; k < NV; k++) red[w][k] = __float2ll_rn(v[k] * FX_SCALE);
		redm[w] = mx;
	}
	__syncthreads();
	if (w == 0) {
#pragma unroll
		for (int k = 0; k < NV; k++) {
			long long s = (int)lane_id() < nw ? red[lane_id()][k] : 0ll;
#pragma unroll
			for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
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
