// dev_decide.cuh - the per-step decision of the device-resident loop.
//
// After each MD step of the graph loop, one warp reads the step's
// accumulator slot and keeps the values; its lane 0 advances the Nose-Hoover alpha for the
// next step (source/sepintgr.c:149-168, from the kinetic sum the step
// produced), applies the skin test of source/sepintgr.c:72 and sets the
// graph's conditional handles (rebuild before the next step; loop on).
// It runs at the end of the fused step kernel, in warp 0 of the block that
// finishes last.
#pragma once
#include "dev_common.cuh"

struct RunState {
	double alpha;          // alpha for the next step
	double alpha_last;     // alpha used by the last completed step
	double sumv2;          // sum m v^2 of the current velocities
	long long remaining;   // loop iterations left
	long long done;        // steps completed
	long long ntrig;       // skin-triggered updates
	long long total;       // steps in this call (the last one produces the observables)
	int force_trig;        // report an update after the next step
	int last_trig;         // the last completed step reported an update
	int abort;
	unsigned arrive;       // blocks of the current step kernel that have finished
	double last[SLOT_FIELDS];
};

struct DecideArgs {
	RunState *rs;          // NULL: no decision in this launch
	long long *slot;
	const unsigned *flags;
	float thr2;            // (skin/2)^2
	double dt_tau2, T0, n;
	int nh;
	int pair_end;          // last step of a loop iteration: count down, set the loop handle
	int use_handles;
	int reset_while;       // first step of an iteration: clear the loop handle on entry
	int obs_all;           // every step is observed (measurement of the API loop's work)
	cudaGraphConditionalHandle h_next, h_while;
};

__device__ __forceinline__ void decide_abort(const DecideArgs &a)
{
	a.rs->abort = 1;
	if (a.use_handles) {
		cudaGraphSetConditional(a.h_next, 0);
		if (a.pair_end) cudaGraphSetConditional(a.h_while, 0);
	}
}

// Hand-over of a step's sums to the host without a copy engine: the
// accumulator slots and the status word are written into pinned host memory
// mapped into the device's address space, then the slots are cleared for
// the next step -- unless keep is set and the status word's overflow bit is
// (a fused step on an overflowed list did nothing, and the slots filled
// before it stay for its second run).  A thread clears only the fields it
// has read itself, so no barrier is needed.
struct TakeArgs {
	long long *h;          // host mirror of the slots (device address); NULL: no hand-over
	unsigned *hf;          // host mirror of the status word (device address)
	unsigned *arrive;      // blocks of the launch that have finished
	long long *slots;
	const unsigned *flags;
	int nread, nall, keep;
};

__device__ __forceinline__ void take_copy(const TakeArgs &t, int tid, int nthr)
{
	const unsigned f0 = __ldcg(t.flags);
	for (int k = tid; k < t.nread * SLOT_FIELDS; k += nthr) t.h[k] = __ldcg(t.slots + k);
	if (tid < 4) t.hf[tid] = __ldcg(t.flags + tid);
	if (t.keep && (f0 & 1u)) return;
	for (int k = tid; k < t.nall * SLOT_FIELDS; k += nthr) t.slots[k] = 0;
}

// At the end of a fused step kernel of the C-API path, after the block's
// accumulator atomics (issued by thread 0): warp 0 of the last block to
// arrive hands the sums over.  Every lane of warp 0 must reach this call.
__device__ __forceinline__ void step_take_exit(const TakeArgs &t)
{
	if (!t.h || threadIdx.x >= 32) return;
	unsigned last = 0;
	if (threadIdx.x == 0) {
		__threadfence();
		last = atomicAdd(t.arrive, 1u) == gridDim.x - 1;
	}
	last = __shfl_sync(0xffffffffu, last, 0);
	if (!last) return;
	__threadfence();
	take_copy(t, threadIdx.x, 32);
	if (threadIdx.x == 0) *t.arrive = 0;
}

// The step skipped its work (overflowed list): no block adds to the slots,
// so warp 0 of block 0 hands over what the slots and the status word hold.
__device__ __forceinline__ void step_take_skip(const TakeArgs &t)
{
	if (t.h && blockIdx.x == 0 && threadIdx.x < 32) take_copy(t, threadIdx.x, 32);
}

// Called by the 32 lanes of one warp: lane k takes accumulator field k
// (SLOT_FIELDS == 32) with one coalesced read; lane 0 then updates the
// thermostat and makes the decision.
__device__ __forceinline__ void decide_warp(const DecideArgs &a)
{
	static_assert(SLOT_FIELDS == 32, "one accumulator field per lane");
	const unsigned FULL = 0xffffffffu;
	const int lane = threadIdx.x & 31;
	RunState *rs = a.rs;
	if (rs->abort || (__ldcg(a.flags) & 1u)) {
		if (lane == 0) decide_abort(a);
		return;
	}
	const long long v = __ldcg(a.slot + lane);
	const double val = (lane == SLOT_MAXD2) ? (double)__uint_as_float((unsigned)v) : (double)v * FX_ISCALE;
	rs->last[lane] = val;
	a.slot[lane] = 0;
	const double sumv2 = __shfl_sync(FULL, val, SLOT_SUMV2);
	const double maxd2 = __shfl_sync(FULL, val, SLOT_MAXD2);
	if (lane != 0) return;
	rs->sumv2 = sumv2;
	rs->alpha_last = rs->alpha;
	if (a.nh) {
		// same operation order and roundings as sep_nosehoover on the host
		// (no contraction), so both paths produce the same alpha bits
		const double ekin = __ddiv_rn(__dmul_rn(0.5, sumv2), a.n);
		const double temp = __dmul_rn(0.666667, ekin);
		rs->alpha = __dadd_rn(rs->alpha, __dmul_rn(a.dt_tau2, __dsub_rn(__ddiv_rn(temp, a.T0), 1.0)));
	}
	const int trig = ((float)maxd2 > a.thr2) || rs->force_trig;
	rs->force_trig = 0;
	rs->last_trig = trig;
	rs->ntrig += trig;
	rs->done += 1;
	if (a.use_handles) {
		cudaGraphSetConditional(a.h_next, trig ? 1u : 0u);
		if (a.pair_end) {
			rs->remaining -= 1;
			cudaGraphSetConditional(a.h_while, rs->remaining > 0 ? 1u : 0u);
		}
	}
}

// Whether this step's energy and virial are observed: in the device loop
// only the last step of a call reports them (sep_gpu_run returns the last
// step's sepret); every other step needs forces, the kinetic sum and the
// displacement only.  Without a decision (API path), or when asked to
// (obs_all), every step reports.
__device__ __forceinline__ bool step_observed(const DecideArgs &a)
{
	return a.obs_all || !a.rs || a.rs->done + 1 >= a.rs->total;
}

// In a step kernel with a decision attached: on entry (before anything can
// return), the first step of a loop iteration clears the loop handle, so the
// loop only goes on when a decision sets it again.
__device__ __forceinline__ void step_decide_entry(const DecideArgs &a)
{
	if (a.rs && a.reset_while && blockIdx.x == 0 && threadIdx.x == 0)
		cudaGraphSetConditional(a.h_while, 0);
}

// The step found the list overflow flag set and skips its work: block 0
// records the abort and stops the loop.
__device__ __forceinline__ void step_decide_skip(const DecideArgs &a)
{
	if (a.rs && blockIdx.x == 0 && threadIdx.x == 0) decide_abort(a);
}

// At the end of the step kernel, after the block's accumulator atomics
// (issued by thread 0): warp 0 of the last block to arrive makes the
// decision.  Every lane of warp 0 must reach this call.
__device__ __forceinline__ void step_decide_exit(const DecideArgs &a)
{
	if (!a.rs || threadIdx.x >= 32) return;
	unsigned last = 0;
	if (threadIdx.x == 0) {
		__threadfence();
		last = atomicAdd(&a.rs->arrive, 1u) == gridDim.x - 1;
	}
	last = __shfl_sync(0xffffffffu, last, 0);
	if (!last) return;
	__threadfence();
	if (threadIdx.x == 0) a.rs->arrive = 0;
	decide_warp(a);
}
