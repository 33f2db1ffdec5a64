// dev_batch.cuh - shared declarations of the batched multi-system path.
//
// Many independent LJ systems share one set of device arrays.  System s
// owns the slots [off, off + npad) (npad = n rounded up to a warp, so every
// warp belongs to one system; slots past n are inert padding) and the cell
// entries [coff, coff + ncell + 2): its real cells, one cell that holds its
// padding, and the end of the last range.  Per-warp and per-cell tables give
// the owning system.
#pragma once
#include <vector>
#include "dev_common.cuh"
#include "dev_decide.cuh"
#include "dev_pair.cuh"

#define SEPB_MAXTYPES 4     // particle types of a typed batch

struct BatchSys {
	int off, n, npad;      // slots and real particles
	int coff, ncell;       // cell offset, real cells
	int nc[3];             // cells per side
	float fs;              // L / 2^32 (cubic box)
	float shi, slo;        // dt * 2^64 / L as a float pair
	LjScale sc;            // the single-LJ constants in this box's units
	int team, groups;      // kernel parameters of the system's size class
	double cellf;          // cell edge over the list cut-off
	double L;
	double T0;             // thermostat target
};

// per-system loop state
struct BatchState {
	double alpha;          // alpha for the next step
	double alpha_last;     // alpha used by the last completed step
	double sumv2;
	long long ntrig;       // skin-triggered updates (the reference's nupdate_neighb)
	int force_trig;        // report an update after the next step
	int last_trig;
	double loss;           // sum of loss_scale * (epot + p) over the steps (adjoint runs)
	double last[SLOT_FIELDS];
};

// loop state shared by all systems
struct BatchRun {
	long long remaining;   // loop iterations left
	long long done;        // steps completed
	long long total;       // steps in this call (the last one reports observables)
	unsigned arrive;       // systems decided in the current step
	unsigned any;          // some system asked for a rebuild in the current step
	unsigned last_any;     // ... in the last completed step
	int abort;
};

struct BatchDecide {
	const BatchSys *sys;
	BatchState *bs;
	BatchRun *run;
	long long *slots;      // SLOT_FIELDS per system
	unsigned *flag;        // per system: rebuild before the next step
	const unsigned *oflow; // list overflow word
	int nsys;
	float thr2;
	double dt_tau2;
	int nh;
	int pair_end, use_handles, reset_while;
	double loss_scale;     // != 0: accumulate the loss term of every step
	cudaGraphConditionalHandle h_next, h_while;
};

// launchers implemented next to the single-system kernels they share code with
int sepdev_batch_step(sepdev *d, const PairArgs &a, const BatchSys *sys, const int4 *wstep, int nwarps,
		      const BatchState *bs, const BatchRun *run, long long *slots, const BatchDecide &dec,
		      int typed);
// perm != NULL: the cell lists hold slot indices (particles not moved);
// fw != NULL: the flagged systems' warps (fcnt of them) to build, else every
// warp of a flagged system
int sepdev_batch_build(sepdev *d, int parity, const int *cellstart, const BatchSys *sys,
		       const int *wsys, int nwarps, const unsigned *flag, float rl2, const int *perm,
		       const int *fw = nullptr, const int *fcnt = nullptr);

// host-side batch (dev_batch.cu); the adjoint (dev_adj.cu) builds on it
struct sepb {
	sepdev *d;                 // the shared per-slot arrays, list, stream
	int nsys;
	long ntot;                 // slots (sum of npad)
	int nwarps;
	long ncells;               // cell entries (sum of ncell + 2)
	double rc, skin, dt, tau;
	int nh;
	double cf, eps, sigma, aw, ushift;
	// typed batch (ntypes > 1): {cf, eps, sigma, aw} per ordered type pair
	// (symmetric), type ids in pos.w
	int ntypes;
	double tparam[SEPB_MAXTYPES * SEPB_MAXTYPES][4];
	std::vector<char> fresh;       // state set and not yet run (types may be set)
	std::vector<BatchSys> hsys;
	BatchSys *sys;             // device
	int *wsys, *csys;
	int4 *wstep;               // per warp of the step kernel: system, first slot, team, groups
	int nstepw;
	unsigned *flag;
	int *fw, *fcnt;            // warps of the flagged systems (kb_compact), for the list build, and their count
	int *cellcount, *cellstart;
	long long *slots;
	BatchState *bs;            // device
	BatchRun *run;
	BatchState *h_bs;          // pinned
	BatchRun *h_run;
	int state_set;             // systems whose state has been set
	std::vector<char> have;
	std::vector<unsigned> nupd;    // list updates since set-up (the reference's nupdate_neighb)
	std::vector<double> alpha0;    // initial thermostat states
	int list_ok;
	// graph of the loop
	cudaGraph_t graph;
	cudaGraphExec_t exec;
	int graph_parity;
	const int *graph_nl;       // list the graph was captured with
	int graph_maxnb;
	// timing
	void *flush_buf;
	size_t flush_bytes;
};

PairArgs batch_pair_args(sepb *b, int parity);
BatchDecide batch_decide_args(sepb *b);
int batch_cells_launch(sepb *b, int parity);
int batch_rebuild_launch(sepb *b, int parity);
int batch_step_launch(sepb *b, int parity, const BatchDecide &dec);
int batch_initial_lists(sepb *b);
int batch_fail(const char *what, int rc);
void batch_to_fixed(double x, double L, unsigned *hi, unsigned *lo);
double batch_from_fixed(unsigned hi, unsigned lo, double L);
