/*
 * sepgpu.h - entry points this GPU implementation adds to the sep C API.
 *
 * None of these has a counterpart in the reference library; the reference
 * hot-path calls keep their meaning (see the other headers).  Programs that
 * only use the reference calls need nothing from this header.
 *
 * Residency.  The particle state of a seppart array lives on the GPU from the
 * first hot-path call on.  The host copy in the array is refreshed at these
 * observation points: sep_eval_mom(), sep_save_xyz(), sep_gpu_sync() and
 * every library call that reads particle data on the host.  The sepret and
 * the sepsys counters are current after every sep_leapfrog().  A program that
 * writes atoms[i].x/v/f/m/z/type directly after the first hot-path call must
 * call sep_gpu_invalidate() before the next library call.
 */
#ifndef SEP_GB300_SEPGPU_H
#define SEP_GB300_SEPGPU_H

#include "sepstrct.h"

#ifdef __cplusplus
extern "C" {
#endif

/* 1 when a CUDA device is usable, else 0. */
int sep_gpu_available(void);

/* Last device error message (empty when none). */
const char *sep_gpu_error(void);

/* Observation point: copy the device state into the seppart array. */
int sep_gpu_sync(seppart *ptr);

/* The seppart array was changed directly on the host: upload it before the
 * next device call. */
int sep_gpu_invalidate(seppart *ptr);

/* Key of the counter-based random streams of sep_force_dpd, sep_fp and
 * sep_langevinGJF (Philox4x32-10; a draw depends on the seed, the user
 * indices it is for and the number of earlier calls of the same function).
 * Setting the seed also restarts those call counts.  0 on success. */
int sep_gpu_set_seed(seppart *ptr, unsigned long long seed);

/*
 * Device-resident MD loop: nsteps repetitions of
 *     sep_reset_retval; sep_reset_force;
 *     sep_force_pairs(types, cf, fun, opt)   (fun != NULL)
 *       or sep_force_lj(types, ljparam, opt) (fun == NULL);
 *     [sep_nosehoover(T0, alpha, tau)]       (nh != 0);
 *     sep_leapfrog;
 * captured once in a CUDA graph whose neighbour-list rebuild is a
 * conditional node decided on the device.  On return ret holds the last
 * step's values, *alpha the thermostat state and sys the counters, exactly as
 * after the equivalent call sequence.  Energy and virial are accumulated on
 * the last step only, since no earlier step's sepret can be read.  Returns 0
 * on success.
 */
int sep_gpu_run(seppart *ptr, sepsys *sys, sepret *ret, const char *types,
		double (*fun)(double, char), const double *ljparam, double cf,
		unsigned opt, int nh, double T0, double *alpha, double tau, long nsteps);

/*
 * Kernel parameters by system size, chosen by the autotuner
 * (seplib_gb300/tune.py: short timed trials on the GPU, cached as JSON) or
 * set by hand.  A system of n particles takes the first class with
 * n <= nmax[k]; the last class takes every larger system.
 *   team    lanes per particle in the Lennard-Jones step kernels, 1 or 2;
 *   groups  groups of four neighbours a lane gathers per iteration, 1 or 2
 *           (a speed choice only: the sums keep their order);
 *   cellf   cell edge of the neighbour-list build over the list cut-off,
 *           1.0 to 2.0.
 * team and cellf change the order of floating-point sums: a system gives
 * the same bits alone (sep_gpu_run, the C API loop) and in a batch
 * (sepbatch.h) under the same table.  A single system takes its class at
 * every neighbour-list build, a batch at sepb_create.  Default: one class,
 * team 1, groups 2, cellf 1.0.  Returns 0, or -1 for values out of range.
 */
#define SEP_GPU_NCLASS 8
typedef struct {
	int nclass;
	long nmax[SEP_GPU_NCLASS];
	int team[SEP_GPU_NCLASS];
	int groups[SEP_GPU_NCLASS];
	double cellf[SEP_GPU_NCLASS];
} sep_gpu_tuning;

int sep_gpu_set_tuning(const sep_gpu_tuning *t);
int sep_gpu_get_tuning(sep_gpu_tuning *t);

/* Diagnostics. */
typedef struct {
	long launches;        /* kernel launches issued for this system */
	long list_builds;     /* neighbour-list builds */
	int list_capacity;    /* neighbour slots per particle */
	int list_max;         /* largest neighbour count of the current list */
	double list_mean;     /* mean neighbour count (full list) */
	int team, groups;     /* kernel parameters taken at the last list build */
	double cellf;
	int direct_io;        /* 1: uploads/downloads read and write the seppart array from
	                       * device code (GPU access to pageable host memory) */
} sep_gpu_info;

int sep_gpu_info_get(seppart *ptr, sep_gpu_info *info);

/* Unordered neighbour pairs (i < j, user indices, sorted) of the current
 * full list; returns the count (pairs filled up to cap), negative on error. */
long sep_gpu_list_pairs(seppart *ptr, int *pairs, long cap);

/* Events on the library's stream, for timing from the caller: record event
 * e (0..7) / elapsed milliseconds between two recorded events. */
int sep_gpu_event_record(seppart *ptr, int e);
int sep_gpu_event_elapsed(seppart *ptr, int e0, int e1, float *ms);
int sep_gpu_stream_sync(seppart *ptr);

/*
 * Timing helper: run nsteps steps of the sep_gpu_run loop from the host
 * (rebuilds outside the timed brackets) and return the mean duration of the
 * fused step kernel in ms, measured with events around each launch.  As with
 * sep_gpu_run, ret reports the last step (energy and virial are only
 * accumulated there).
 */
int sep_gpu_time_step_kernel(seppart *ptr, sepsys *sys, sepret *ret, const char *types,
			     double (*fun)(double, char), const double *ljparam, double cf,
			     unsigned opt, int nh, double T0, double *alpha, double tau,
			     long nsteps, double *ms_per_launch);

/*
 * Timing helper: sep_gpu_run's loop (same arguments, same results) arranged
 * for measurement.  Before every step the library writes tm->flush_bytes to
 * a buffer of its own (on its stream, outside the timed spans) so that no
 * step finds the previous step's data in L2.  One pair of CUDA events per
 * step brackets either the whole step (list rebuild when due, fused
 * force + integration kernel, loop decision) or, with kernel_spans 1, the
 * fused kernel alone; the summed device times come back in tm.  With
 * kernel_spans 2 nothing is flushed and the events bracket whole launches of
 * up to 64 steps (for working sets larger than L2, where a flush adds
 * nothing but the events' own cost).
 */
typedef struct {
	long flush_bytes;      /* in: bytes written between steps (0: no flush) */
	int kernel_spans;      /* in: 0: time each step; 1: time each fused step kernel;
				* 2: time whole launches of up to 64 steps, with no event
				* inside them (flush_bytes must be 0) */
	double ms_steps;       /* out: summed device time of the steps (kernel_spans == 0) */
	double ms_kernel;      /* out: summed device time of the kernels (kernel_spans == 1) */
	long launches;         /* out: steps launched */
	long overflows;        /* out: neighbour-list regrowths (outside the spans) */
	int observe;           /* in: 1: every step sums its energy and virial, as a loop of
				* API calls does; 0: only the last step, as sep_gpu_run */
} sep_gpu_timing;

int sep_gpu_run_timed(seppart *ptr, sepsys *sys, sepret *ret, const char *types,
		      double (*fun)(double, char), const double *ljparam, double cf, unsigned opt,
		      int nh, double T0, double *alpha, double tau, long nsteps, sep_gpu_timing *tm);

/* Write `bytes` to a library-owned device buffer on the library's stream and
 * wait for it: evicts the L2 cache between timed calls. */
int sep_gpu_flush_l2(seppart *ptr, long bytes);

/*
 * Lennard-Jones forces for callers that may not allocate device memory.
 * No counterpart in the reference: it is an addition of this library.
 *
 * Who needs it: host programs that give all device memory to their own pool
 * allocator at start-up and forbid any allocation outside it, and loops
 * where the device-wide synchronisation of cudaMalloc/cudaFree is too
 * costly.  This call allocates nothing (no cudaMalloc, no library routine
 * that allocates): its working memory is a fixed array of about 5 MB inside
 * the library, sized for at most 131072 particles and 65536 linked cells
 * (cells of edge >= cf per box side).  Larger inputs return an error before
 * any work is issued.
 *
 * It computes what sep_force_lj computes for one particle type and SEP_ALL:
 * param = {cf, eps, sigma, aw} (as in sep_force_lj), shifted so the pair
 * energy is zero at cf.  x (3n doubles, x0 y0 z0 x1 ...) is read from device
 * memory; f (3n doubles, overwritten, not added to) and *epot (the total pair
 * energy) are written to device memory.  L (3 box lengths) and param are
 * host arrays.  All work is queued on `stream` (a cudaStream_t; NULL is the
 * legacy default stream) and the call returns without waiting.
 *
 * The cut-off param[0] may be at most half the shortest box side; larger
 * cut-offs are rejected.
 *
 * The fixed array is shared by every call and keeps the last call's
 * contents; each call clears what it needs.  Calls whose work overlaps on
 * the GPU (different streams, or several host threads) race on it and give
 * wrong results: order them on one stream.  The first call on each device,
 * with that device current, looks up the array's address and keeps it.
 * Under CUDA's default lazy module loading, that first call is also when
 * the array (and the code it runs) is placed on the device: the first call
 * takes about 5 MB of device memory, later calls take none.  So make the
 * first call before a pool allocator takes the device's memory, and before
 * any stream capture.  Particles are binned with atomics, so the summation
 * order of a particle's pair terms, and with it the last bits of the
 * results, can differ from call to call.
 *
 * Returns 0, or a negative code with the message in sep_gpu_error().
 */
int sep_gpu_lj_forces_noalloc(const double *x, long n, const double *L, const double *param,
			      double *f, double *epot, void *stream);

#ifdef __cplusplus
}
#endif
#endif
