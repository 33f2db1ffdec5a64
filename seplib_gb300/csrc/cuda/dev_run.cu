// dev_run.cu - device-resident multi-step loop in one CUDA graph.
//
// The loop body holds RUN_UNROLL MD steps (an even number, so the
// double-buffered positions return to the same buffer and every captured
// argument stays valid):
//
//   WHILE (iterations left) {
//     IF (rebuild 0) { sort + list build from buffer p }
//     fused step p -> p^1, deciding at its end (sets IF 1)
//     IF (rebuild 1) { sort + list build from buffer p^1 }
//     fused step p^1 -> p, deciding (sets IF 2)
//     ...
//     fused step, deciding (sets IF 0, counts down, sets WHILE)
//   }
//
// The decision (dev_decide.cuh) is made by the block of the fused step kernel
// that finishes last: it reads the step's accumulator slot, advances the
// Nose-Hoover alpha, applies the skin test and sets the conditional handles.
// The first step of every iteration clears the WHILE handle on entry, so the
// loop only continues when the last decision of the iteration sets it again.
// No host round trip happens inside the loop.  A neighbour-list overflow
// inside the loop makes the following step kernels skip and the loop stop;
// the host grows the list and resumes.  Steps beyond a multiple of
// RUN_UNROLL run one at a time from the host.
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "dev_common.cuh"
#include "dev_pair.cuh"

#define RUN_UNROLL 8

int sepdev_sort_async(sepdev *d, int parity, int trigger);
int sepdev_build_async(sepdev *d, int parity);
int sepdev_grow_list(sepdev *d, int needed);
int sepdev_upload_pairset(sepdev *d, const sepdev_pairset *ps);

struct Runner {
	cudaGraph_t graph;
	cudaGraphExec_t exec;
	RunState *rs;          // device
	RunState *h_rs;        // pinned
	// key of the captured graph
	sepdev_pairset ps;
	double dt, T0, tau, skin;
	int nh, parity, maxnb, team, groups;
	const int *nl;
	long ncells;
	int valid;
};

void sepdev_runner_free(sepdev *d)
{
	Runner *r = (Runner *)d->runner;
	if (!r) return;
	if (r->exec) cudaGraphExecDestroy(r->exec);
	if (r->graph) cudaGraphDestroy(r->graph);
	if (r->rs) cudaFree(r->rs);
	if (r->h_rs) cudaFreeHost(r->h_rs);
	free(r);
	d->runner = NULL;
}

static int runner_get(sepdev *d, Runner **out)
{
	if (!d->runner) {
		Runner *r = (Runner *)calloc(1, sizeof(Runner));
		if (!r) return SEPDEV_ENOMEM;
		d->runner = r;
		CK(cudaMalloc((void **)&r->rs, sizeof(RunState)));
		CK(cudaMallocHost((void **)&r->h_rs, sizeof(RunState)));
	}
	*out = (Runner *)d->runner;
	return SEPDEV_OK;
}

static DecideArgs decide_args(sepdev *d, Runner *r, const sepdev_runcfg *cfg)
{
	DecideArgs a;
	memset(&a, 0, sizeof a);
	a.rs = r->rs;
	a.slot = d->slots;
	a.flags = d->flags;
	a.thr2 = (float)(0.25 * cfg->skin * cfg->skin);
	a.dt_tau2 = cfg->dt / (cfg->tau * cfg->tau);
	a.T0 = cfg->T0;
	a.n = (double)d->n;
	a.nh = cfg->nh;
	a.obs_all = cfg->observe_all;
	return a;
}

// one fused step from buffer `parity`, deciding at its end
static int step_launch(sepdev *d, Runner *r, const sepdev_pairset *ps, const sepdev_runcfg *cfg,
		       int parity, const DecideArgs &dec)
{
	PairArgs a;
	sepdev_fill_args(d, a, ps, cfg->dt, cfg->nh, 0.0, 0, 0, 0, parity);
	a.alpha_dev = &r->rs->alpha;
	a.flags = d->flags;
	a.dec = dec;
	return sepdev_launch_pair(d, ps, a, true);
}

static int rebuild_launch(sepdev *d, int parity)
{
	int rc = sepdev_sort_async(d, parity, 1);
	if (rc) return rc;
	return sepdev_build_async(d, parity);
}

// add an IF node to `g` after `dep` and capture the rebuild into it
static int add_if_rebuild(sepdev *d, cudaGraph_t g, const cudaGraphNode_t *dep, int ndep,
			  cudaGraphConditionalHandle h, int parity, cudaGraphNode_t *out)
{
	cudaGraphNodeParams p = {cudaGraphNodeTypeConditional};
	p.conditional.handle = h;
	p.conditional.type = cudaGraphCondTypeIf;
	p.conditional.size = 1;
	CK(cudaGraphAddNode(out, g, dep, NULL, ndep, &p));
	cudaGraph_t body = p.conditional.phGraph_out[0];
	CK(cudaStreamBeginCaptureToGraph(d->st, body, NULL, NULL, 0, cudaStreamCaptureModeRelaxed));
	int rc = rebuild_launch(d, parity);
	cudaGraph_t tmp;
	cudaError_t e = cudaStreamEndCapture(d->st, &tmp);
	if (rc) return rc;
	if (e != cudaSuccess) { sepdev_set_error("capture(rebuild)", e); return SEPDEV_ECUDA; }
	return SEPDEV_OK;
}

// the node the next captured operation on d->st would depend on
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

static int end_capture(sepdev *d, int rc, cudaError_t e, const char *what)
{
	cudaGraph_t tmp;
	cudaError_t e2 = cudaStreamEndCapture(d->st, &tmp);
	if (rc) return rc;
	if (e != cudaSuccess || e2 != cudaSuccess) {
		sepdev_set_error(what, e != cudaSuccess ? e : e2);
		return SEPDEV_ECUDA;
	}
	return SEPDEV_OK;
}

// capture one fused step into `g` after node `dep`; *last = its node
static int add_step(sepdev *d, Runner *r, cudaGraph_t g, cudaGraphNode_t dep,
		    const sepdev_pairset *ps, const sepdev_runcfg *cfg, int parity,
		    const DecideArgs &dec, cudaGraphNode_t *last)
{
	CK(cudaStreamBeginCaptureToGraph(d->st, g, &dep, NULL, 1, cudaStreamCaptureModeRelaxed));
	int rc = step_launch(d, r, ps, cfg, parity, dec);
	if (!rc) rc = capture_tail(d, last);
	return end_capture(d, rc, cudaSuccess, "capture(step)");
}

static int build_graph(sepdev *d, Runner *r, const sepdev_pairset *ps, const sepdev_runcfg *cfg,
		       int parity)
{
	if (r->exec) { cudaGraphExecDestroy(r->exec); r->exec = NULL; }
	if (r->graph) { cudaGraphDestroy(r->graph); r->graph = NULL; }
	r->valid = 0;
	CK(cudaGraphCreate(&r->graph, 0));
	cudaGraphConditionalHandle hw, hif[RUN_UNROLL];
	CK(cudaGraphConditionalHandleCreate(&hw, r->graph, 1, cudaGraphCondAssignDefault));
	for (int k = 0; k < RUN_UNROLL; k++)
		CK(cudaGraphConditionalHandleCreate(&hif[k], r->graph, 0, cudaGraphCondAssignDefault));
	cudaGraphNodeParams wp = {cudaGraphNodeTypeConditional};
	wp.conditional.handle = hw;
	wp.conditional.type = cudaGraphCondTypeWhile;
	wp.conditional.size = 1;
	cudaGraphNode_t wnode;
	CK(cudaGraphAddNode(&wnode, r->graph, NULL, NULL, 0, &wp));
	cudaGraph_t body = wp.conditional.phGraph_out[0];
	cudaGraphNode_t tail = NULL;
	int rc;
	for (int k = 0; k < RUN_UNROLL; k++) {
		cudaGraphNode_t nif;
		if ((rc = add_if_rebuild(d, body, k ? &tail : NULL, k ? 1 : 0, hif[k], parity ^ (k & 1), &nif)))
			return rc;
		DecideArgs dec = decide_args(d, r, cfg);
		dec.use_handles = 1;
		dec.h_next = hif[(k + 1) % RUN_UNROLL];
		dec.h_while = hw;
		dec.reset_while = (k == 0);
		dec.pair_end = (k == RUN_UNROLL - 1);
		if ((rc = add_step(d, r, body, nif, ps, cfg, parity ^ (k & 1), dec, &tail))) return rc;
	}
	CK(cudaGraphInstantiate(&r->exec, r->graph, 0));
	r->ps = *ps;
	r->dt = cfg->dt; r->T0 = cfg->T0; r->tau = cfg->tau; r->skin = cfg->skin; r->nh = cfg->nh;
	r->parity = parity; r->maxnb = d->maxnb; r->team = d->team; r->groups = d->groups; r->nl = d->nl;
	r->ncells = d->ncells;
	r->valid = 1;
	return SEPDEV_OK;
}

static bool graph_matches(const sepdev *d, const Runner *r, const sepdev_pairset *ps,
			  const sepdev_runcfg *cfg, int parity)
{
	return r->valid && r->parity == parity && r->maxnb == d->maxnb && r->team == d->team &&
	       r->groups == d->groups &&
	       r->nl == d->nl && r->ncells == d->ncells && r->dt == cfg->dt && r->T0 == cfg->T0 &&
	       r->tau == cfg->tau && r->skin == cfg->skin && r->nh == cfg->nh &&
	       memcmp(&r->ps, ps, sizeof *ps) == 0;
}

// the state at the start of a call: alpha already advanced for the first step
static int run_begin(sepdev *d, Runner *r, const sepdev_pairset *ps, const sepdev_runcfg *cfg,
		     double alpha, double sumv2, long nsteps)
{
	int rc = sepdev_upload_pairset(d, ps);
	if (rc) return rc;
	RunState *h = r->h_rs;
	memset(h, 0, sizeof *h);
	h->sumv2 = sumv2;
	h->alpha = alpha;
	h->alpha_last = alpha;
	h->force_trig = cfg->force_trigger;
	h->total = nsteps;
	CK(cudaMemsetAsync(d->slots, 0, sizeof(long long) * SLOT_FIELDS, d->st));
	CK(cudaMemsetAsync(d->flags, 0, sizeof(unsigned) * 2, d->st));
	return SEPDEV_OK;
}

// neighbour-list overflow inside the loop: grow, rebuild, clear the abort
static int run_recover(sepdev *d, RunState *h)
{
	unsigned fl[2];
	CK(cudaMemcpy(fl, d->flags, sizeof fl, cudaMemcpyDeviceToHost));
	int rc;
	if ((rc = sepdev_grow_list(d, (int)fl[1]))) return rc;
	if ((rc = sepdev_build_list(d, d->rlist, d->excl, 1))) return rc;
	h->abort = 0;
	h->last_trig = 0;
	return SEPDEV_OK;
}

static void run_end(const RunState *h, double *alpha, double *sumv2, double *last, long *ntrig,
		    int *last_trig)
{
	*alpha = h->alpha_last;
	*sumv2 = h->sumv2;
	if (last) memcpy(last, h->last, sizeof(double) * SLOT_FIELDS);
	if (ntrig) *ntrig = h->ntrig;
	if (last_trig) *last_trig = h->last_trig;
}

static int run_loop(sepdev *d, const sepdev_pairset *ps, const sepdev_runcfg *cfg,
		    long nsteps, double *alpha, double *sumv2, double *last, long *ntrig,
		    int *last_trig)
{
	if (!d->list_valid || nsteps < 0) return SEPDEV_EINVAL;
	int rc;
	if ((rc = sepdev_list_confirm(d))) return rc;
	Runner *r;
	rc = runner_get(d, &r);
	if (rc) return rc;
	if ((rc = run_begin(d, r, ps, cfg, *alpha, *sumv2, nsteps))) return rc;
	RunState *h = r->h_rs;
	int recoveries = 0;
	while (h->done < nsteps) {
		const long todo = nsteps - h->done;
		const long done0 = h->done;
		if (todo >= RUN_UNROLL) {
			h->remaining = todo / RUN_UNROLL;
			CK(cudaMemcpyAsync(r->rs, h, sizeof *h, cudaMemcpyHostToDevice, d->st));
			if (!graph_matches(d, r, ps, cfg, d->cur) && (rc = build_graph(d, r, ps, cfg, d->cur)))
				return rc;
			CK(cudaGraphLaunch(r->exec, d->st));
			d->launches++;
		} else {
			// a step outside the graph (fewer than RUN_UNROLL left)
			if (h->last_trig && (rc = sepdev_build_list(d, d->rlist, d->excl, 1))) return rc;
			h->remaining = 0;
			CK(cudaMemcpyAsync(r->rs, h, sizeof *h, cudaMemcpyHostToDevice, d->st));
			if ((rc = step_launch(d, r, ps, cfg, d->cur, decide_args(d, r, cfg)))) return rc;
		}
		CK(cudaMemcpyAsync(h, r->rs, sizeof *h, cudaMemcpyDeviceToHost, d->st));
		CK(cudaStreamSynchronize(d->st));
		// every completed step flipped the position buffer
		if ((h->done - done0) & 1) d->cur ^= 1;
		if (h->abort) {
			if (++recoveries > 16) return SEPDEV_EOVERFLOW;
			if ((rc = run_recover(d, h))) return rc;
		}
	}
	run_end(h, alpha, sumv2, last, ntrig, last_trig);
	return SEPDEV_OK;
}

// The loop graphs carry no molecular-tensor sums: those are kept off while
// they are captured and launched.
extern "C" int sepdev_run(sepdev *d, const sepdev_pairset *ps, const sepdev_runcfg *cfg,
			  long nsteps, double *alpha, double *sumv2, double *last, long *ntrig,
			  int *last_trig)
{
	const int mv = d->molvir_on;
	d->molvir_on = 0;
	const int rc = run_loop(d, ps, cfg, nsteps, alpha, sumv2, last, ntrig, last_trig);
	d->molvir_on = mv;
	return rc;
}

// ---- timed loop: L2 flushed between steps, events around every step -------
//
// The same device work as the loop above, organised for measurement.  One
// graph holds TM_RING steps unrolled (or the remainder of the run):
//
//   setif (first IF from the previous step's decision) ->
//   { flush -> [e0] IF (rebuild) -> fused step, deciding [e1] } x S
//
// The flush writes flush_bytes to a context-owned buffer so that no step
// finds the previous step's data in L2; it lies outside the [e0, e1] span.
// With kernel_spans 1 the events bracket the fused step kernel instead of
// the whole step; with kernel_spans 2 there are no events inside the graph
// and no flush: one pair of stream events brackets each graph launch.  The
// host launches one graph per TM_RING steps and reads the events between
// launches.

#define TM_RING 64

__global__ void k_setif(const RunState *rs, cudaGraphConditionalHandle h)
{
	if (threadIdx.x == 0 && blockIdx.x == 0)
		cudaGraphSetConditional(h, (rs->last_trig && !rs->abort) ? 1u : 0u);
}

__global__ void k_flush(uint4 *buf, long n16, unsigned tag)
{
	for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n16; i += (long)gridDim.x * blockDim.x)
		buf[i] = make_uint4((unsigned)i, tag, (unsigned)i ^ tag, 0u);
}

static int flush_reserve(sepdev *d, size_t bytes)
{
	if (d->flush_bytes >= bytes) return SEPDEV_OK;
	if (d->flush_buf) { CK(cudaFree(d->flush_buf)); d->flush_buf = NULL; d->flush_bytes = 0; }
	CK(cudaMalloc(&d->flush_buf, bytes));
	d->flush_bytes = bytes;
	return SEPDEV_OK;
}

static void flush_launch(sepdev *d, size_t bytes, unsigned tag)
{
	k_flush<<<d->nsm * 4, 512, 0, d->st>>>((uint4 *)d->flush_buf, (long)(bytes / 16), tag);
}

extern "C" int sepdev_flush_l2(sepdev *d, size_t bytes, unsigned tag)
{
	bytes &= ~(size_t)15;
	if (bytes == 0) return SEPDEV_OK;
	int rc = flush_reserve(d, bytes);
	if (rc) return rc;
	flush_launch(d, bytes, tag);
	CKL(d);
	return SEPDEV_OK;
}

struct TimedEvents {
	cudaEvent_t e0[TM_RING], e1[TM_RING];
	int made;
};

static void timed_events_free(TimedEvents *t)
{
	for (int j = 0; j < t->made; j++) {
		cudaEventDestroy(t->e0[j]);
		cudaEventDestroy(t->e1[j]);
	}
	t->made = 0;
}

static int timed_events_make(TimedEvents *t)
{
	t->made = 0;
	for (int j = 0; j < TM_RING; j++) {
		CK(cudaEventCreate(&t->e0[j]));
		cudaError_t e = cudaEventCreate(&t->e1[j]);
		if (e != cudaSuccess) {
			cudaEventDestroy(t->e0[j]);
			sepdev_set_error("cudaEventCreate", e);
			return SEPDEV_ECUDA;
		}
		t->made = j + 1;
	}
	return SEPDEV_OK;
}

struct TimedGraph {
	cudaGraph_t g;
	cudaGraphExec_t exec;
	int nsteps, parity;
};

static void timed_graph_free(TimedGraph *t)
{
	if (t->exec) cudaGraphExecDestroy(t->exec);
	if (t->g) cudaGraphDestroy(t->g);
	memset(t, 0, sizeof *t);
}

static int build_timed_graph(sepdev *d, Runner *r, const sepdev_pairset *ps, const sepdev_runcfg *cfg,
			     int parity, int nsteps, size_t flush, int kernel_spans,
			     const TimedEvents *ev, TimedGraph *t)
{
	CK(cudaGraphCreate(&t->g, 0));
	t->nsteps = nsteps;
	t->parity = parity;
	cudaGraphConditionalHandle h[TM_RING];
	for (int k = 0; k < nsteps; k++)
		CK(cudaGraphConditionalHandleCreate(&h[k], t->g, 0, cudaGraphCondAssignDefault));
	cudaGraphNode_t tail;
	int rc = SEPDEV_OK;
	cudaError_t e = cudaSuccess;
	CK(cudaStreamBeginCaptureToGraph(d->st, t->g, NULL, NULL, 0, cudaStreamCaptureModeRelaxed));
	k_setif<<<1, 32, 0, d->st>>>(r->rs, h[0]);
	rc = capture_tail(d, &tail);
	if ((rc = end_capture(d, rc, e, "capture(setif)"))) return rc;
	for (int k = 0; k < nsteps; k++) {
		const int p = parity ^ (k & 1);
		CK(cudaStreamBeginCaptureToGraph(d->st, t->g, &tail, NULL, 1, cudaStreamCaptureModeRelaxed));
		if (flush) flush_launch(d, flush, 0x9e3779b9u * (unsigned)(k + 1));
		if (kernel_spans == 0) e = cudaEventRecordWithFlags(ev->e0[k], d->st, cudaEventRecordExternal);
		if (e == cudaSuccess) rc = capture_tail(d, &tail);
		if ((rc = end_capture(d, rc, e, "capture(flush)"))) return rc;
		cudaGraphNode_t nif;
		if ((rc = add_if_rebuild(d, t->g, &tail, 1, h[k], p, &nif))) return rc;
		CK(cudaStreamBeginCaptureToGraph(d->st, t->g, &nif, NULL, 1, cudaStreamCaptureModeRelaxed));
		DecideArgs dec = decide_args(d, r, cfg);
		if (k + 1 < nsteps) {
			dec.use_handles = 1;
			dec.h_next = h[k + 1];
		}
		if (kernel_spans == 1) e = cudaEventRecordWithFlags(ev->e0[k], d->st, cudaEventRecordExternal);
		if (e == cudaSuccess) rc = step_launch(d, r, ps, cfg, p, dec);
		if (e == cudaSuccess && !rc && kernel_spans != 2)
			e = cudaEventRecordWithFlags(ev->e1[k], d->st, cudaEventRecordExternal);
		if (e == cudaSuccess && !rc) rc = capture_tail(d, &tail);
		if ((rc = end_capture(d, rc, e, "capture(timed step)"))) return rc;
	}
	CK(cudaGraphInstantiate(&t->exec, t->g, 0));
	return SEPDEV_OK;
}

static int run_timed_inner(sepdev *d, Runner *r, const sepdev_pairset *ps, const sepdev_runcfg *cfg,
			   long nsteps, sepdev_timing *tm, TimedEvents *ev, TimedGraph tg[2])
{
	RunState *h = r->h_rs;
	const size_t flush = (size_t)(tm->flush_bytes > 0 ? tm->flush_bytes : 0) & ~(size_t)15;
	// kernel_spans 2: one span per graph launch, so no flush may sit inside it
	const bool whole = tm->kernel_spans == 2;
	if (whole && flush) return SEPDEV_EINVAL;
	int rc;
	if (flush && (rc = flush_reserve(d, flush))) return rc;
	CK(cudaMemcpyAsync(r->rs, h, sizeof *h, cudaMemcpyHostToDevice, d->st));
	while (h->done < nsteps) {
		const long left = nsteps - h->done;
		const int m = (int)(left < TM_RING ? left : TM_RING);
		// tg[0]: full rings, tg[1]: the remainder; rebuilt when the key changes
		TimedGraph *t = &tg[m == TM_RING ? 0 : 1];
		if (t->exec && (t->nsteps != m || t->parity != d->cur)) timed_graph_free(t);
		if (!t->exec &&
		    (rc = build_timed_graph(d, r, ps, cfg, d->cur, m, flush, tm->kernel_spans, ev, t)))
			return rc;
		const long done0 = h->done;
		if (whole) CK(cudaEventRecord(ev->e0[0], d->st));
		CK(cudaGraphLaunch(t->exec, d->st));
		if (whole) CK(cudaEventRecord(ev->e1[0], d->st));
		d->launches += 1;
		CK(cudaMemcpyAsync(h, r->rs, sizeof *h, cudaMemcpyDeviceToHost, d->st));
		CK(cudaStreamSynchronize(d->st));
		double sum = 0.0;
		for (int j = 0; j < (whole ? 1 : m); j++) {
			float a = 0.f;
			CK(cudaEventElapsedTime(&a, ev->e0[j], ev->e1[j]));
			sum += a;
		}
		if (tm->kernel_spans == 1) tm->ms_kernel += sum;
		else tm->ms_steps += sum;
		tm->launches += m;
		// every completed step flipped the position buffer
		if ((h->done - done0) & 1) d->cur ^= 1;
		if (h->abort) {
			// the rest of this graph skipped its work: grow and rebuild
			// outside the timed spans, then go on
			if (tm->overflows >= 16) return SEPDEV_EOVERFLOW;
			timed_graph_free(&tg[0]);
			timed_graph_free(&tg[1]);
			if ((rc = run_recover(d, h))) return rc;
			CK(cudaMemsetAsync(d->flags, 0, sizeof(unsigned) * 2, d->st));
			CK(cudaMemcpyAsync(r->rs, h, sizeof *h, cudaMemcpyHostToDevice, d->st));
			tm->overflows += 1;
		}
	}
	return SEPDEV_OK;
}

static int run_timed_loop(sepdev *d, const sepdev_pairset *ps, const sepdev_runcfg *cfg,
			  long nsteps, double *alpha, double *sumv2, double *last, long *ntrig,
			  int *last_trig, sepdev_timing *tm);

extern "C" int sepdev_run_timed(sepdev *d, const sepdev_pairset *ps, const sepdev_runcfg *cfg,
				long nsteps, double *alpha, double *sumv2, double *last, long *ntrig,
				int *last_trig, sepdev_timing *tm)
{
	const int mv = d->molvir_on;
	d->molvir_on = 0;
	const int rc = run_timed_loop(d, ps, cfg, nsteps, alpha, sumv2, last, ntrig, last_trig, tm);
	d->molvir_on = mv;
	return rc;
}

static int run_timed_loop(sepdev *d, const sepdev_pairset *ps, const sepdev_runcfg *cfg,
			  long nsteps, double *alpha, double *sumv2, double *last, long *ntrig,
			  int *last_trig, sepdev_timing *tm)
{
	if (!d->list_valid || nsteps < 0 || !tm) return SEPDEV_EINVAL;
	if (sepdev_list_confirm(d)) return SEPDEV_ECUDA;
	tm->ms_steps = tm->ms_kernel = 0.0;
	tm->launches = 0;
	tm->overflows = 0;
	Runner *r;
	int rc = runner_get(d, &r);
	if (rc) return rc;
	if ((rc = run_begin(d, r, ps, cfg, *alpha, *sumv2, nsteps))) return rc;
	TimedEvents *ev = (TimedEvents *)calloc(1, sizeof(TimedEvents));
	if (!ev) return SEPDEV_ENOMEM;
	TimedGraph tg[2];
	memset(tg, 0, sizeof tg);
	rc = timed_events_make(ev);
	if (!rc) rc = run_timed_inner(d, r, ps, cfg, nsteps, tm, ev, tg);
	cudaStreamSynchronize(d->st);
	timed_graph_free(&tg[0]);
	timed_graph_free(&tg[1]);
	timed_events_free(ev);
	free(ev);
	if (rc) return rc;
	run_end(r->h_rs, alpha, sumv2, last, ntrig, last_trig);
	return SEPDEV_OK;
}
