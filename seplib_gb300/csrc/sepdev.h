/*
 * sepdev.h - C ABI between the C99 host layer (the csrc/host sources) and the
 * CUDA device layer (the csrc/cuda sources).  Plain pointers and sizes only.
 *
 * One sepdev context holds one particle system resident on the GPU:
 *   - positions as 64-bit fixed-point fractions of the box edge, split in a
 *     32-bit high word (packed with the type id in an int4, double-buffered,
 *     read by the pair kernels) and a 32-bit low word;
 *   - velocities as float-float pairs (hi + lo), mass and 1/mass packed in the
 *     fourth lanes;
 *   - forces as float4 (xyz + per-particle pair energy);
 *   - everything stored in cell order (a spatial sort refreshed at every
 *     neighbour-list build), with gid[] mapping a slot to the user index.
 * Reductions (energies, virial, kinetic tensor) land in "slots" of 64-bit
 * fixed-point accumulators (scale 2^32), read back in one copy.
 */
#ifndef SEPDEV_H
#define SEPDEV_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sepdev sepdev;

/* status codes (0 = success) */
#define SEPDEV_OK            0
#define SEPDEV_ECUDA        -1   /* CUDA runtime error, message in sepdev_last_error() */
#define SEPDEV_ENOMEM       -2
#define SEPDEV_EINVAL       -3
#define SEPDEV_EOVERFLOW    -4   /* neighbour list capacity exceeded */
#define SEPDEV_ENODEV       -5   /* no CUDA device */

#define SEPDEV_MAXTYPES 16

/* stochastic-dynamics per-particle fields (sepdev_ext_*) */
enum { SEPDEV_EXT_PV = 0, SEPDEV_EXT_PA = 1, SEPDEV_EXT_PREVF = 2, SEPDEV_EXT_RANDN = 3,
       SEPDEV_NEXT = 4 };
#define SEPDEV_MAXCHAN   4

/* fields of one accumulator slot (int64, value * 2^32) */
enum {
	SLOT_EPOT0 = 0,        /* energy channels 0..3 */
	SLOT_ECOUL = 4,
	SLOT_POTP = 5,         /* pot_P: 6 entries xx xy xz yy yz zz (9 reserved) */
	SLOT_POTPB = 14,       /* pot_P_bond: 6 entries (9 reserved) */
	SLOT_EKIN = 23,        /* sum m vt^2 (leap-frog kinetic term, before the 1/2) */
	SLOT_KINP = 24,        /* 6 entries xx xy xz yy yz zz */
	SLOT_SUMV2 = 30,       /* sum m v^2 after the step (for the next Nose-Hoover call) */
	SLOT_MAXD2 = 31,       /* max squared displacement since the last build, float bits */
	SLOT_FIELDS = 32
};

/* exclusion modes for the list build (see the oracle's ora_excluded) */
enum { SEPDEV_EXCL_NONE = 0, SEPDEV_EXCL_BONDS = 1, SEPDEV_EXCL_ALLBONDED = 2,
       SEPDEV_EXCL_SAMEMOL = 3 };

/* pair-potential kinds */
enum { SEPDEV_POT_OFF = 0, SEPDEV_POT_LJ = 1, SEPDEV_POT_TABLE = 2 };

/*
 * Pair interaction table for one force pass: for every ordered type pair
 * (ti, tj) one potential.  LJ: ft = eps48 s6 (s6 - awh) sig2/r^2 with
 * s6 = (sig2/r^2)^3, u = eps4 s6 (s6 - aw) + ushift, cut at rc2.
 * TABLE: tabulated ft(r^2) and u(r^2) on a uniform r^2 grid.
 */
typedef struct {
	int kind;
	int chan;              /* energy channel 0..3 */
	float rc2;
	float eps48, eps4, sig2, aw, awh;
	float ushift;
	float ushl;            /* the shift's remainder: shift - (float)shift */
	int table;             /* index of the table for SEPDEV_POT_TABLE */
} sepdev_pot;

typedef struct {
	int ntypes;
	int nchan;                                  /* energy channels in use */
	sepdev_pot pot[SEPDEV_MAXTYPES * SEPDEV_MAXTYPES];
	int coulomb;                                /* shifted-force Coulomb on */
	float coul_rc2, coul_irc2, coul_irc, coul_rc;
} sepdev_pairset;

/* ---- context ---- */
int sepdev_create(sepdev **out, long n);
void sepdev_destroy(sepdev *d);
const char *sepdev_last_error(void);
int sepdev_device_count(void);

/*
 * Upload the full state (user order).  x, v: 3n doubles; m, z: n doubles;
 * type_id, molindex: n ints; crossings, cross_neighb: 3n ints; L: 3 doubles.
 * The internal order is reset to the user order and the list marked stale.
 */
int sepdev_upload(sepdev *d, const double *x, const double *v, const double *f,
		  const double *m, const double *z, const int *type_id, const int *molindex,
		  const int *crossings, const int *cross_neighb, const double *L);

/* Download to user order.  Any pointer may be NULL.  xn receives the
 * positions at the last list build. */
int sepdev_download(sepdev *d, double *x, double *v, double *f, int *crossings,
		    int *cross_neighb, double *xn);

/*
 * In-place transfers: the device reads and writes the seppart array itself
 * (parts = the program's seppart pointer, n records).  Available when the GPU
 * can address pageable host memory (sepdev_direct_io != 0).  The upload also
 * returns the type characters in order of first appearance (at most
 * max_types, ids 0..*ntypes-1), sum m v^2 (FP64, fixed summation order) and
 * the largest squared displacement from the records' xn; more than
 * max_types characters give SEPDEV_EOVERFLOW.  The download
 * writes x, v, f (zero when forces_zero), a = f/m, crossings, cross_neighb
 * and xn.
 */
int sepdev_direct_io(const sepdev *d);
int sepdev_upload_parts(sepdev *d, const void *parts, const double *L, int max_types,
			char *tchar, int *ntypes, double *sumv2, double *maxd2);
int sepdev_download_parts(sepdev *d, void *parts, int forces_zero);

/* Sum of m v^2 over the current velocities (one reduction, synchronous). */
int sepdev_sumv2(sepdev *d, double *out);

/* Exclusion partner lists in user order: two CSR tables, partners by user
 * index; `bonds` = direct bonds, `all` = bond+angle+dihedral partners. */
int sepdev_set_exclusions(sepdev *d, const int *bond_start, const int *bond_idx,
			  const int *all_start, const int *all_idx);

/* Tabulated potential: nt points, ft and u at r2 = r2min + k*dr2. */
int sepdev_set_table(sepdev *d, int table, int nt, double r2min, double dr2,
		     const float *ft, const float *u);

/* ---- accumulator slots ---- */
int sepdev_slots_reset(sepdev *d);              /* zero all slots (async) */
/* Synchronous: out[nslots*SLOT_FIELDS] as doubles (MAXD2 decoded), flags =
 * status word; then all slots are zeroed, except when keep_on_overflow is
 * set and flags[0] & 1 (a deferred step that skipped its work). */
int sepdev_slots_take(sepdev *d, int nslots, double *out, unsigned *flags, int keep_on_overflow);

/* ---- neighbour list ---- */
/* Rebuild the cell order and the full neighbour list with cut-off rlist.
 * trigger != 0 marks a skin-triggered rebuild (crossing base reset). */
int sepdev_build_list(sepdev *d, double rlist, int excl, int trigger);
/* The same without waiting for the capacity check: the list is marked
 * unchecked.  sepdev_step_deferred runs on it (skipping its work if the
 * build overflowed), sepdev_slots_take settles it when its flags show no
 * overflow, every other consumer confirms it first (synchronous). */
int sepdev_build_list_deferred(sepdev *d, double rlist, int excl, int trigger);
int sepdev_list_confirm(sepdev *d);
/* Pair set of the current list, user indices, i<j, unique: returns count,
 * fills up to cap pairs (2 ints each).  Test and diagnostics helper. */
long sepdev_list_pairs(sepdev *d, int *pairs, long cap);
int sepdev_list_stats(sepdev *d, int *maxcount, double *meancount, int *capacity);

/* ---- forces and integration ---- */
/*
 * Pair forces of `ps` over the current list.  accumulate != 0 adds to the
 * stored forces, otherwise overwrites them.  Energies go to slot `slot`
 * channels, virial to its POTP entries.
 */
int sepdev_pair_forces(sepdev *d, const sepdev_pairset *ps, int accumulate, int slot);

/*
 * Leap-frog (source/sepintgr.c:42-88 semantics) on the stored forces.
 * nh != 0 subtracts alpha m v first and stores the modified force.
 * Kinetic terms, sum m v^2 and the displacement maximum go to `slot`.
 */
int sepdev_leapfrog(sepdev *d, double dt, int nh, double alpha, int slot);

/* Fused pair forces + optional Nose-Hoover friction + leap-frog in one kernel. */
int sepdev_step(sepdev *d, const sepdev_pairset *ps, int accumulate, double dt,
		int nh, double alpha, int pair_slot, int lf_slot);
/* the same with observe = 0: the pair slot receives no energy or virial (a
 * step of a loop whose sepret only reports its last step) */
int sepdev_step_obs(sepdev *d, const sepdev_pairset *ps, int accumulate, double dt,
		    int nh, double alpha, int pair_slot, int lf_slot, int observe);

/* sepdev_step on a list that may be unchecked (sepdev_build_list_deferred);
 * if flags[0] & 1 at the following sepdev_slots_take, the step did nothing:
 * sepdev_step_retract, sepdev_list_confirm, and run it again.  take_n >= 0:
 * the step kernel itself hands slots [0, take_n) and the flags to the host
 * at its end, and the next sepdev_slots_take (which must ask for take_n
 * slots, with keep_on_overflow) only waits for it. */
int sepdev_step_deferred(sepdev *d, const sepdev_pairset *ps, int accumulate, double dt,
			 int nh, double alpha, int pair_slot, int lf_slot, int take_n);
void sepdev_step_retract(sepdev *d);

/* f -= alpha m v on the stored forces. */
int sepdev_friction(sepdev *d, double alpha);

/* Set stored forces to zero. */
int sepdev_zero_forces(sepdev *d);

/* ---- bonded terms ---- */
/* Topology in user indices: nb bonds (a,b,type), na angles (a,b,c,type),
 * nd dihedrals (a,b,c,d,type). */
int sepdev_set_topology(sepdev *d, int nb, const unsigned *blist, int na,
			const unsigned *alist, int nd, const unsigned *dlist);
/* Bonded terms, up to one of each kind per launch: kind 0 bonds (p0 = l0,
 * p1 = k; energy, pot_P and pot_P_bond to the term's slot), 1 angles
 * (p0 = theta0, p1 = k, cossq: the cos^2 form; energy), 2 Ryckaert-Bellemans
 * torsions (g; energy).  The forces are added to the stored ones
 * (accumulate) or stored. */
typedef struct {
	int kind, type;
	double p0, p1;
	int cossq;
	double g[6];
	int slot;
} sepdev_bterm;
int sepdev_bonded(sepdev *d, const sepdev_bterm *t, int nt, int accumulate);
/* per-term observables of the last call of each kind (0 bond lengths,
 * 1 angles, 2 dihedral angles), in topology order */
int sepdev_term_values(sepdev *d, int kind, double *out);

/* ---- timing and multi-step ---- */
int sepdev_sync(sepdev *d);
/* events on the context stream: record into slot e (0..7), elapsed ms */
int sepdev_event_record(sepdev *d, int e);
int sepdev_event_elapsed(sepdev *d, int e0, int e1, float *ms);

/*
 * Run nsteps of {pair forces, [Nose-Hoover], leap-frog} entirely on the
 * device, rebuilding the list when the skin test fires.  The loop is one
 * CUDA graph (WHILE node over eight unrolled steps, each behind an IF node
 * that holds the captured list rebuild); at the end of each fused step the
 * last block to finish updates the thermostat and decides the rebuild.
 * Steps beyond a multiple of eight run singly.  The list must be valid on
 * entry.  alpha: in, the thermostat value the first step uses (already
 * advanced by the caller); out, the value the last step used, as
 * sep_nosehoover leaves it; sumv2: sum m v^2 in/out; last: the final step's
 * slot values (SLOT_FIELDS doubles); ntrig: skin-triggered updates;
 * last_trig: whether the final step requested an update.
 */
typedef struct {
	double dt, skin;
	int nh;
	double T0, tau;
	int force_trigger;     /* report an update after the first step */
	int observe_all;       /* every step sums its energy and virial (else only the last) */
} sepdev_runcfg;

int sepdev_run(sepdev *d, const sepdev_pairset *ps, const sepdev_runcfg *cfg, long nsteps,
	       double *alpha, double *sumv2, double *last, long *ntrig, int *last_trig);

/*
 * The same loop for measurement: graphs of up to 64 unrolled steps with an
 * L2 flush of flush_bytes before every step, outside the timed spans, and
 * one pair of CUDA events per step (around the step, or around its fused
 * step kernel).  Results and outputs as sepdev_run.
 */
typedef struct {
	long flush_bytes;      /* in: bytes written between steps (0: no flush) */
	int kernel_spans;      /* in: 0: events around each step; 1: around each fused step kernel;
				* 2: around each graph launch of up to 64 steps (no flush) */
	double ms_steps;       /* out: summed device time of the steps (kernel_spans == 0) */
	double ms_kernel;      /* out: summed device time of the fused step kernel (kernel_spans == 1) */
	long launches;         /* out: steps launched (skipped ones included) */
	long overflows;        /* out: list overflows recovered outside the spans */
} sepdev_timing;

int sepdev_run_timed(sepdev *d, const sepdev_pairset *ps, const sepdev_runcfg *cfg, long nsteps,
		     double *alpha, double *sumv2, double *last, long *ntrig, int *last_trig,
		     sepdev_timing *tm);

/* queue a write of `bytes` (rounded down to 16) to a context-owned buffer */
int sepdev_flush_l2(sepdev *d, size_t bytes, unsigned tag);

/* ---- samplers (dev_sampler.cu) ----
 * vacf: a device ring of lvec rows of x-velocities by user index; _store
 * fills row index from the current state, _block returns C[k] = sum_i sum_kk
 * v[kk][i] v[k+kk][i] for k < lvec (host array).  msd: _base keeps the
 * current unwrapped positions and crossing counts; _sample returns (host,
 * 2 + nk) sum |dr|^2, sum |dr|^4 and sum cos(k_j dr_x) over particles of
 * type id type_id.  FP64, fixed summation order. */
typedef struct sepdev_vacf sepdev_vacf;
typedef struct sepdev_msd sepdev_msd;
int sepdev_vacf_create(sepdev *d, int lvec, sepdev_vacf **out);
void sepdev_vacf_destroy(sepdev_vacf *v);
int sepdev_vacf_store(sepdev *d, sepdev_vacf *v, int index);
int sepdev_vacf_block(sepdev *d, sepdev_vacf *v, double *out);
/* radial distribution: out[b * ncomb + c] = the number of pairs i < j with
 * floor(r / dg) = b (dg = L_x / (2 lvec)) whose type ids (ti, tj) have bit c
 * set in mask[ti * nt + tj] (ncomb <= 32, lvec * ncomb <= 49152) */
int sepdev_radial(sepdev *d, int lvec, int ncomb, int nt, const unsigned *mask, double *out);
/* atomic generalised hydrodynamics: per wavevector k[j] along y (unwrapped
 * by the crossings), out[15 j + 2 q + (0 re, 1 im)] = sum over particles of
 * e^{i k_j y} w_q with w = (m, m v_x, m v_y, m v^2/2, 1, m a_y, m v_y^2),
 * a = f / m of the stored forces; out[15 j + 14] = sum m v^2/2 */
typedef struct sepdev_gh sepdev_gh;
int sepdev_gh_create(sepdev *d, int nk, const double *k, sepdev_gh **out);
void sepdev_gh_destroy(sepdev_gh *g);
int sepdev_gh_sample(sepdev *d, sepdev_gh *g, double *out);
/* partial coherent scattering: per wavevector k_j = 2 pi (j+1) / L_x, per
 * requested type u (umap: device type id -> u or -1) and class c (nclass
 * 1: all particles; 2: even molecule index, odd or no molecule) the sum of
 * m e^{i k_j x} (x unwrapped): out[j * 2 nu nclass + 2 (u nclass + c) + (0
 * re, 1 im)]; 2 nu nclass <= 28 */
int sepdev_scatt(sepdev *d, int nk, int nu, int nclass, const int *umap, double *out);
/* a ring of count values per sample (mvacf: one per molecule) */
int sepdev_vacf_create_count(sepdev *d, int lvec, long count, sepdev_vacf **out);
double *sepdev_vacf_row(sepdev_vacf *v, int index);
long sepdev_vacf_count(const sepdev_vacf *v);

/* Per-type operations.  _set_x0: tether positions (user order, 3 n
 * doubles); _tether: f += k (x0 - x) (minimum image) on the particles of
 * type id tid; _type_sums: out[0..2] sum m v, out[3] sum m, out[4] sum m v^2,
 * out[5] count over the type; _type_scale: v = v fact - shift on the type;
 * _profile: lvec bins of L_dir / lvec along dir over the type, out[4 b + q]
 * = sum m v[dirvel], sum m, sum m v^2 over the other two components, count
 * (4 lvec doubles; lvec <= 1536). */
int sepdev_set_x0(sepdev *d, const double *x0);
int sepdev_tether(sepdev *d, int tid, double k);
int sepdev_type_sums(sepdev *d, int tid, double *out);
int sepdev_type_scale(sepdev *d, int tid, double fact, const double *shift);
int sepdev_profile(sepdev *d, int tid, int dir, int dirvel, int lvec, double *out);

/* Molecule tables of the molecular samplers: first atom and length of each
 * molecule's chain of consecutive user indices (centres of mass), its atoms
 * as CSR over user indices, molecule masses. */
typedef struct sepdev_moltab sepdev_moltab;
int sepdev_moltab_create(sepdev *d, int nmol, const int *first, const int *nuau, const int *start,
			 const int *atoms, const double *mass, sepdev_moltab **out);
void sepdev_moltab_destroy(sepdev_moltab *t);
/* mvacf: the molecules' centre-of-mass x-velocities into row index of a
 * ring created with count nmol */
int sepdev_mvacf_store(sepdev *d, sepdev_moltab *t, sepdev_vacf *v, int index);
/* mavacf: the type-A molecules' (sel) end-to-end y component (atom 0 to
 * atom b) times q times the molecule mass into row index of a ring created
 * with count nmol */
int sepdev_mavacf_store(sepdev *d, sepdev_moltab *t, sepdev_vacf *v, int index, const unsigned char *sel,
			int b, double q);
/* mgh: for each wavevector k[j] along y, out[18 j + 2 q + (0 re, 1 im)] =
 * sum over molecules of e^{i k_j y_cm} w_q with w = (M, M vx, M vy, M v^2/2,
 * 1, s_z, s_y, dipole_y, w_x) (w_x, the angular velocity, only when unsafe;
 * else 0); out[18 nk] = sum of M v^2/2.  The dipole of a molecule without
 * both signs of charge keeps its last value (initially 0). */
int sepdev_mgh_sample(sepdev *d, sepdev_moltab *t, int nk, const double *k, int unsafe, double *out);
/* Molecular mean square displacement: sel (host, nmol) marks the
 * molecules of the sampled type, reset starts a block (the centres of mass
 * become the reference and the crossing counts restart); out (host, 1 + nk)
 * = sum |dr|^2 and sum cos(k_j dr_x) over the marked molecules. */
typedef struct sepdev_mmsd sepdev_mmsd;
int sepdev_mmsd_create(sepdev *d, sepdev_moltab *t, int nk, const double *k, sepdev_mmsd **out);
void sepdev_mmsd_destroy(sepdev_mmsd *m);
int sepdev_mmsd_sample(sepdev *d, sepdev_moltab *t, sepdev_mmsd *m, const unsigned char *sel, int reset,
		       double *out);
/* Molecular profiles: over the molecules marked in sel (host, nmol),
 * binned by the centre of mass along dir into lvec bins, out[16 b + q]
 * (host) = sum m v[dirvel], m, count, spin (3), m v^2 over the other two
 * components, inertia tensor (9, row-major). */
int sepdev_mprofs(sepdev *d, sepdev_moltab *t, const unsigned char *sel, int dir, int dirvel, int lvec,
		  double *out);
/* Molecular Berendsen step along z: each molecule's centre-of-mass z is
 * scaled by `scale` and its atoms keep their offsets from it, the box edge
 * L_z becomes L1z; atoms outside molecules keep their absolute z. */
int sepdev_berendsen_mol(sepdev *d, sepdev_moltab *t, double L1z, double scale);
int sepdev_msd_create(sepdev *d, int nk, const double *k, sepdev_msd **out);
void sepdev_msd_destroy(sepdev_msd *m);
int sepdev_msd_base(sepdev *d, sepdev_msd *m);
int sepdev_msd_sample(sepdev *d, sepdev_msd *m, int type_id, double *out);

/* ---- stochastic dynamics (dev_stoch.cu) ----
 * _ext_enable allocates the SEPDEV_EXT_* fields (zero); _ext_upload and
 * _ext_download move them in user order (3 n doubles each, ldiff n
 * doubles; any pointer may be NULL to skip a field).  Random numbers come
 * from Philox4x32-10 keyed by `seed`: a DPD pair draws from the counter
 * (min gid, max gid, call, 1), a particle of sep_fp / GJF from
 * (gid, 0, call, 2 / 3).  Each integrator writes its kinetic sums (m v^2,
 * m v v^T of the updated velocities), sum m v^2 and the displacement
 * maximum into `slot`. */
typedef struct {
	int tA, tB;              /* type ids of the pair (-1: absent) */
	double cf, aij, gamma, sigma, dt;
	unsigned long long seed;
	unsigned call;
	int virial;              /* 1: pot_P (conservative) to slot, random and
	                          * dissipative parts to slot2 (the O(N^2) form) */
	int mslot;               /* with virial and the molecular tensor on: the
	                          * slot of the conservative forces' molecular
	                          * sums (as a pair pass's); -1 none */
} sepdev_dpd;
int sepdev_ext_enable(sepdev *d);
int sepdev_ext_enabled(const sepdev *d);
int sepdev_ext_upload(sepdev *d, const double *pv, const double *pa, const double *prevf,
		      const double *randn, const double *ldiff);
int sepdev_ext_download(sepdev *d, double *pv, double *pa, double *prevf, double *randn);
/* DPD pair forces added to (accumulate) or stored into the forces; the
 * energy sum aij w^2 / 2 into slot's channel 0 */
int sepdev_dpd_forces(sepdev *d, const sepdev_dpd *p, int accumulate, int slot, int slot2);
int sepdev_verlet_dpd(sepdev *d, double dt, double lambda, int stepnow, int slot);
int sepdev_fp(sepdev *d, double dt, double temp, unsigned long long seed, unsigned call, int slot);
int sepdev_gjf(sepdev *d, double dt, double temp, double alpha, unsigned long long seed,
	       unsigned call, int slot);

/* ---- box changes (dev_box.cu) ----
 * New box edges L1; every position coordinate k is multiplied by sx[k]
 * (in FP64) and re-expressed in the new box, wrapped with its crossing
 * counted; the last-update positions keep their absolute values. */
int sepdev_rescale_box(sepdev *d, const double *L1, const double *sx);

/* ---- molecular pressure tensor (dev_molp.cu) ----
 * _enable: nmol molecules; first/nuau: the chain of consecutive user indices
 * the centre of mass is taken over; start/atoms: each molecule's atoms
 * (CSR, user indices); mass: molecule masses.  While enabled every pair pass
 * computes the centres of mass of its positions and accumulates the
 * molecular virial and the per-atom intermolecular force; _slot names the
 * slot that receives the pass's molecular sums (fields 0-8: sum f (x) R_ij;
 * 9-17: sum f (x) n_ij, n_ij the periodic image of R_ij).  _reset zeroes the
 * per-atom forces.  _state returns kin (9: sum M v v^T), corr (9:
 * sum_i F_i (x) dR_i, dR_i = L1 f1_i - L0 f0_i the change of the centre of
 * mass since the last pass in the box of each time), and each molecule's
 * centre of mass (3 nmol, wrapped) and velocity (3 nmol); the current and
 * the pass's box are returned in L1 and L0 (3 each, may be NULL). */
int sepdev_molvir_enable(sepdev *d, int nmol, const int *first, const int *nuau, const int *start,
			 const int *atoms, const double *mass);
int sepdev_molvir_reset(sepdev *d);
int sepdev_molvir_slot(sepdev *d, int slot);
void sepdev_molvir_disable(sepdev *d);
int sepdev_mol_state(sepdev *d, double *kin, double *corr, double *cm, double *vcm, double *L0,
		     double *L1);

/*
 * Kernel parameters by system size, the table the autotuner fills (one per
 * process).  A system of n particles takes the first class with n <=
 * nmax[k] (the last class takes every larger system):
 *   team    lanes per particle in the LJ step kernels (1 or 2);
 *   groups  groups of four neighbours each lane gathers per iteration
 *           (1 or 2; only a speed choice, the sums keep their order);
 *   cellf   cell edge of the list build over the list cut-off (1 to 2).
 * team and cellf change the order of floating-point sums, so one system
 * gives the same bits alone and in a batch only under the same table.  A
 * single system takes its class at every list build; a batch at creation.
 */
#define SEPDEV_NCLASS 8
typedef struct {
	int nclass;
	long nmax[SEPDEV_NCLASS];
	int team[SEPDEV_NCLASS];
	int groups[SEPDEV_NCLASS];
	double cellf[SEPDEV_NCLASS];
} sepdev_tuning;
int sepdev_tuning_set(const sepdev_tuning *t);      /* SEPDEV_EINVAL if out of range */
void sepdev_tuning_get(sepdev_tuning *t);
void sepdev_tuning_for(long n, int *team, int *groups, double *cellf);
/* the parameters a context took at its last list build */
void sepdev_params(sepdev *d, int *team, int *groups, double *cellf);

/* kernel launches issued by this context so far (all kinds) */
long sepdev_launch_count(sepdev *d);

#ifdef __cplusplus
}
#endif
#endif
