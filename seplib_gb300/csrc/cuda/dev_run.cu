// dev_run.cu - device-resident multi-step loop in one CUDA graph.
//
// The loop body holds two MD steps (so the double-buffered positions return
// to the same buffer and every captured argument stays valid):
//
//   WHILE (pairs left) {
//     IF (rebuild A) { sort + list build from buffer p }
//     fused step p -> p^1 ; decide A (sets IF B)
//     IF (rebuild B) { sort + list build from buffer p^1 }
//     fused step p^1 -> p ; decide B (sets IF A, counts down, sets WHILE)
//   }
//
// "decide" is a one-thread kernel that reads the step's accumulator slot,
// keeps the last step's values, updates the Nose-Hoover alpha for the next
// step (source/sepintgr.c:149-168, from the kinetic sum the step kernel
// produced), applies the skin test of source/sepintgr.c:72 and sets the
// conditional handles.  No host round trip happens inside the loop.
// A neighbour-list overflow inside the loop makes the next step kernel skip
// and the loop stop; the host grows the list and resumes.
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "dev_common.cuh"
#include "dev_pair.cuh"

int sepdev_sort_async(sepdev *d, int parity, int trigger);
int sepdev_build_async(sepdev *d, int parity);
int sepdev_grow_list(sepdev *d, int needed);
int sepdev_upload_pairset(sepdev *d, const sepdev_pairset *ps);

struct RunState {
	double alpha;          // alpha for the next step
	double alpha_last;     // alpha used by the last completed step
	double sumv2;          // sum m v^2 of the current velocities
	long long remaining;   // loop iterations (step pairs) left
	long long done;        // steps completed
	long long ntrig;       // skin-triggered updates
	int force_trig;        // report an update after the next step
	int last_trig;         // the last completed step reported an update
	int abort;
	int pad;
	double last[SLOT_FIELDS];
};

struct DecideArgs {
	RunState *rs;
	long long *slot;
	const unsigned *flags;
	float thr2;            // (skin/2)^2
	double dt_tau2, T0, n;
	int nh;
	int pair_end;
	int use_handles;
	cudaGraphConditionalHandle h_next, h_while;
};

__global__ void k_decide(DecideArgs a)
{
	if (threadIdx.x != 0 || blockIdx.x != 0) return;
	RunState *rs = a.rs;
	if (rs->abort || (a.flags[0] & 1u)) {
		rs->abort = 1;
		if (a.use_handles) {
			cudaGraphSetConditional(a.h_next, 0);
			if (a.pair_end) cudaGraphSetConditional(a.h_while, 0);
		}
		return;
	}
	for (int k = 0; k < SLOT_FIELDS; k++) {
		const long long v = a.slot[k];
		rs->last[k] = (k == SLOT_MAXD2) ? (double)__uint_as_float((unsigned)v) : (double)v * FX_ISCALE;
		a.slot[k] = 0;
	}
	rs->sumv2 = rs->last[SLOT_SUMV2];
	rs->alpha_last = rs->alpha;
	if (a.nh) {
		// same operation order and roundings as sep_nosehoover on the host
		// (no contraction), so both paths produce the same alpha bits
		const double ekin = __ddiv_rn(__dmul_rn(0.5, rs->sumv2), a.n);
		const double temp = __dmul_rn(0.666667, ekin);
		rs->alpha = __dadd_rn(rs->alpha, __dmul_rn(a.dt_tau2, __dsub_rn(__ddiv_rn(temp, a.T0), 1.0)));
	}
	const int trig = ((float)rs->last[SLOT_MAXD2] > a.thr2) || rs->force_trig;
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

struct Runner {
	cudaGraph_t graph;
	cudaGraphExec_t exec;
	RunState *rs;          // device
	RunState *h_rs;        // pinned
	// key of the captured graph
	sepdev_pairset ps;
	double dt, T0, tau, skin;
	int nh, parity, maxnb, tpp;
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

static int launch_decide(sepdev *d, const DecideArgs &a)
{
	k_decide<<<1, 32, 0, d->st>>>(a);
	CKL(d);
	return SEPDEV_OK;
}

static DecideArgs decide_args(sepdev *d, Runner *r, const sepdev_runcfg *cfg, int pair_end,
			      int use_handles, cudaGraphConditionalHandle hn,
			      cudaGraphConditionalHandle hw)
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
	a.pair_end = pair_end;
	a.use_handles = use_handles;
	a.h_next = hn;
	a.h_while = hw;
	return a;
}

static int step_launch(sepdev *d, Runner *r, const sepdev_pairset *ps, const sepdev_runcfg *cfg,
		       int parity)
{
	PairArgs a;
	sepdev_fill_args(d, a, ps, cfg->dt, cfg->nh, 0.0, 0, 0, 0, parity);
	a.alpha_dev = &r->rs->alpha;
	a.flags = d->flags;
	return sepdev_launch_pair(d, ps, a, true);
}

static int rebuild_launch(sepdev *d, int parity)
{
	int rc = sepdev_sort_async(d, parity, 1);
	if (rc) return rc;
	return sepdev_build_async(d, parity);
}

// capture helpers: add an IF node to `g` after `dep` and capture the rebuild into it
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

// capture step + decide into `g` after node `dep`; returns the last node
static int add_step(sepdev *d, Runner *r, cudaGraph_t g, cudaGraphNode_t dep,
		    const sepdev_pairset *ps, const sepdev_runcfg *cfg, int parity,
		    const DecideArgs &da, cudaGraphNode_t *last)
{
	CK(cudaStreamBeginCaptureToGraph(d->st, g, &dep, NULL, 1, cudaStreamCaptureModeRelaxed));
	int rc = step_launch(d, r, ps, cfg, parity);
	if (!rc) rc = launch_decide(d, da);
	cudaStreamCaptureStatus st;
	const cudaGraphNode_t *deps = NULL;
	size_t nd = 0;
	cudaError_t e = cudaStreamGetCaptureInfo(d->st, &st, NULL, NULL, &deps, NULL, &nd);
	if (e == cudaSuccess && nd >= 1) *last = deps[0];
	cudaGraph_t tmp;
	cudaError_t e2 = cudaStreamEndCapture(d->st, &tmp);
	if (rc) return rc;
	if (e != cudaSuccess || nd < 1) { sepdev_set_error("capture info", e); return SEPDEV_ECUDA; }
	if (e2 != cudaSuccess) { sepdev_set_error("capture(step)", e2); return SEPDEV_ECUDA; }
	return SEPDEV_OK;
}

static int build_graph(sepdev *d, Runner *r, const sepdev_pairset *ps, const sepdev_runcfg *cfg,
		       int parity)
{
	if (r->exec) { cudaGraphExecDestroy(r->exec); r->exec = NULL; }
	if (r->graph) { cudaGraphDestroy(r->graph); r->graph = NULL; }
	CK(cudaGraphCreate(&r->graph, 0));
	cudaGraphConditionalHandle hw, ha, hb;
	CK(cudaGraphConditionalHandleCreate(&hw, r->graph, 1, cudaGraphCondAssignDefault));
	CK(cudaGraphConditionalHandleCreate(&ha, r->graph, 0, cudaGraphCondAssignDefault));
	CK(cudaGraphConditionalHandleCreate(&hb, r->graph, 0, cudaGraphCondAssignDefault));
	cudaGraphNodeParams wp = {cudaGraphNodeTypeConditional};
	wp.conditional.handle = hw;
	wp.conditional.type = cudaGraphCondTypeWhile;
	wp.conditional.size = 1;
	cudaGraphNode_t wnode;
	CK(cudaGraphAddNode(&wnode, r->graph, NULL, NULL, 0, &wp));
	cudaGraph_t body = wp.conditional.phGraph_out[0];
	cudaGraphNode_t ifa, ifb, la, lb;
	int rc;
	if ((rc = add_if_rebuild(d, body, NULL, 0, ha, parity, &ifa))) return rc;
	DecideArgs da = decide_args(d, r, cfg, 0, 1, hb, hw);
	if ((rc = add_step(d, r, body, ifa, ps, cfg, parity, da, &la))) return rc;
	if ((rc = add_if_rebuild(d, body, &la, 1, hb, parity ^ 1, &ifb))) return rc;
	DecideArgs db = decide_args(d, r, cfg, 1, 1, ha, hw);
	if ((rc = add_step(d, r, body, ifb, ps, cfg, parity ^ 1, db, &lb))) return rc;
	CK(cudaGraphInstantiate(&r->exec, r->graph, 0));
	r->ps = *ps;
	r->dt = cfg->dt; r->T0 = cfg->T0; r->tau = cfg->tau; r->skin = cfg->skin; r->nh = cfg->nh;
	r->parity = parity; r->maxnb = d->maxnb; r->tpp = d->tpp; r->nl = d->nl;
	r->ncells = d->ncells;
	r->valid = 1;
	return SEPDEV_OK;
}

static bool graph_matches(const sepdev *d, const Runner *r, const sepdev_pairset *ps,
			  const sepdev_runcfg *cfg, int parity)
{
	return r->valid && r->parity == parity && r->maxnb == d->maxnb && r->tpp == d->tpp &&
	       r->nl == d->nl && r->ncells == d->ncells && r->dt == cfg->dt && r->T0 == cfg->T0 &&
	       r->tau == cfg->tau && r->skin == cfg->skin && r->nh == cfg->nh &&
	       memcmp(&r->ps, ps, sizeof *ps) == 0;
}

extern "C" int sepdev_run(sepdev *d, const sepdev_pairset *ps, const sepdev_runcfg *cfg,
			  long nsteps, double *alpha, double *sumv2, double *last, long *ntrig,
			  int *last_trig)
{
	if (!d->list_valid || nsteps < 0) return SEPDEV_EINVAL;
	if (!d->runner) {
		Runner *r = (Runner *)calloc(1, sizeof(Runner));
		if (!r) return SEPDEV_ENOMEM;
		d->runner = r;
		CK(cudaMalloc((void **)&r->rs, sizeof(RunState)));
		CK(cudaMallocHost((void **)&r->h_rs, sizeof(RunState)));
	}
	Runner *r = (Runner *)d->runner;
	int rc0 = sepdev_upload_pairset(d, ps);
	if (rc0) return rc0;
	RunState *h = r->h_rs;
	memset(h, 0, sizeof *h);
	h->sumv2 = *sumv2;
	h->alpha = *alpha;
	h->alpha_last = *alpha;   // the caller passes alpha already advanced for the first step
	h->force_trig = cfg->force_trigger;
	long todo = nsteps;
	long ntrig_total = 0;
	int rc;
	CK(cudaMemsetAsync(d->slots, 0, sizeof(long long) * SLOT_FIELDS, d->st));
	CK(cudaMemsetAsync(d->flags, 0, sizeof(unsigned) * 2, d->st));
	while (todo > 0) {
		h->remaining = todo / 2;
		h->done = 0;
		h->ntrig = 0;
		h->abort = 0;
		CK(cudaMemcpyAsync(r->rs, h, sizeof *h, cudaMemcpyHostToDevice, d->st));
		if (todo >= 2) {
			if (!graph_matches(d, r, ps, cfg, d->cur) && (rc = build_graph(d, r, ps, cfg, d->cur)))
				return rc;
			CK(cudaGraphLaunch(r->exec, d->st));
			d->launches++;
		}
		CK(cudaMemcpyAsync(h, r->rs, sizeof *h, cudaMemcpyDeviceToHost, d->st));
		CK(cudaStreamSynchronize(d->st));
		if (todo >= 2) {
			// an even number of steps completed leaves the positions in buffer cur
			if (h->done & 1) d->cur ^= 1;
		}
		todo -= h->done;
		ntrig_total += h->ntrig;
		if (h->abort) {
			// list overflow during an in-loop rebuild: grow, rebuild, resume
			unsigned fl[2];
			CK(cudaMemcpy(fl, d->flags, sizeof fl, cudaMemcpyDeviceToHost));
			if ((rc = sepdev_grow_list(d, (int)fl[1]))) return rc;
			if ((rc = sepdev_build_list(d, d->rlist, d->excl, 1))) return rc;
			h->last_trig = 0;
			continue;
		}
		if (todo == 1) {
			// the odd last step outside the graph
			if (h->last_trig) {
				if ((rc = sepdev_build_list(d, d->rlist, d->excl, 1))) return rc;
			}
			h->remaining = 0;
			h->done = 0;
			h->ntrig = 0;
			CK(cudaMemcpyAsync(r->rs, h, sizeof *h, cudaMemcpyHostToDevice, d->st));
			if ((rc = step_launch(d, r, ps, cfg, d->cur))) return rc;
			DecideArgs a1 = decide_args(d, r, cfg, 0, 0, 0, 0);
			if ((rc = launch_decide(d, a1))) return rc;
			CK(cudaMemcpyAsync(h, r->rs, sizeof *h, cudaMemcpyDeviceToHost, d->st));
			CK(cudaStreamSynchronize(d->st));
			d->cur ^= 1;
			todo -= h->done;
			ntrig_total += h->ntrig;
			if (h->abort) return SEPDEV_EOVERFLOW;
		}
	}
	*alpha = h->alpha_last;
	*sumv2 = h->sumv2;
	if (last) memcpy(last, h->last, sizeof(double) * SLOT_FIELDS);
	if (ntrig) *ntrig = ntrig_total;
	if (last_trig) *last_trig = h->last_trig;
	return SEPDEV_OK;
}
