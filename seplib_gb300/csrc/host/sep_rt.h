/*
 * sep_rt.h - host runtime behind the sep C API (internal).
 *
 * Every particle array returned by sep_init()/sep_init_xyz() owns one
 * runtime context, found from the seppart pointer.  The context keeps the
 * particle state resident on the GPU and decides when the host copy in the
 * seppart array and the device copy must be synchronised:
 *
 *   host_valid  the seppart array holds the current x, v, f, crossings, xn
 *   dev_valid   the device holds the current state
 *
 * Hot-path calls run on the device and clear host_valid; calls that read
 * particle data on the host (sep_eval_mom, sep_save_xyz, ...) download
 * first; calls that change particle data on the host (sep_set_lattice,
 * sep_set_vel_seed, topology reading, ...) clear dev_valid so the next
 * device call uploads.
 *
 * Pair-force calls are deferred: the pair terms of one step are gathered and
 * evaluated in a single pass over the neighbour list, fused with the
 * Nose-Hoover friction and the leap-frog when sep_leapfrog() follows.  Any
 * call that needs the forces earlier (bonded terms, observation points)
 * launches the pending pass first.
 *
 * Contributions to a sepret are recorded as an ordered list of operations on
 * device accumulator slots and applied to the caller's sepret in call order
 * when the slots are read back (at the end of every sep_leapfrog, or at an
 * observation point), which reproduces the reference's mix of assigned and
 * accumulated energies exactly.
 */
#ifndef SEP_RT_H
#define SEP_RT_H

#include "sep.h"
#include "sepgpu.h"
#include "../sepdev.h"

#define RT_MAXOPS 128
#define RT_MAXTERMS 4

enum {
	OP_PAIR_ASSIGN = 1,  /* epot  = E[chan]                         (sep_force_pairs) */
	OP_PAIR_ADD,         /* epot += E[chan]                         (sep_force_lj) */
	OP_VIRIAL,           /* pot_P += P                              (every pair pass) */
	OP_COUL,             /* epot += Ec, ecoul += Ec                 (sep_coulomb_sf) */
	OP_BOND,             /* epot += E0, pot_P += P, pot_P_bond += P (stretch) */
	OP_EADD,             /* epot += E0                              (angles, torsions) */
	OP_KIN,              /* ekin += Ek/2, kin_P += K                (leap-frog) */
	OP_DPD_VIR,          /* pot_P, pot_P_conservative += C; pot_P_random += R;
	                      * pot_P_dissipative += D (chan: slot of D) (O(N^2) DPD) */
	OP_MOLVIR            /* context molW += W, molN += N (molecular sums of a pass) */
};

typedef struct {
	sepret *ret;
	int kind;
	int slot;
	int chan;
} rt_op;

typedef struct {
	char t0, t1;        /* type pair */
	int kind;           /* SEPDEV_POT_LJ or SEPDEV_POT_TABLE */
	double rc, eps, sigma, aw, ushift;
	int table;
} rt_term;

typedef struct rt_ctx {
	seppart *ptr;
	long n;
	sepdev *dev;
	int host_valid, dev_valid;

	/* type map */
	char tchar[SEPDEV_MAXTYPES];
	int ntypes;

	/* neighbour-list bookkeeping */
	int list_stale;
	int list_excl;          /* SEPDEV_EXCL_* of the current list */
	double list_rlist;
	int trigger_next;       /* next build is a skin-triggered one */
	int pending_trigger;    /* report an update at the next leap-frog (xn never set) */
	double brute_cf;        /* largest cut-off requested under SEP_BRUTE */

	/* deferred work */
	rt_term terms[RT_MAXTERMS];
	int nterms;
	int coul_on;
	double coul_cf;
	int pass_slot;          /* slot of the pending pair pass, -1 if none */
	int mv_slot;            /* its molecular sums' slot (molecular tensor on) */
	int forces_zero;        /* stored forces are logically zero */
	int x0_valid;           /* the device holds the tether positions x0 */
	sepdev_bterm bq[3];     /* pending bonded terms, at most one per kind */
	int nbq;
	int friction;           /* Nose-Hoover friction pending */
	double friction_alpha;

	/* accumulator slots and recorded operations */
	int nslots;
	rt_op ops[RT_MAXOPS];
	int nops;

	/* sum m v^2 of the current velocities (for Nose-Hoover) */
	double sumv2;
	int sumv2_valid;

	/* topology */
	int topo_dirty;
	int has_topo;
	sepsys *topo_sys;       /* the system whose molptr holds the lists */

	/* tabulated user potentials */
	double (*tab_fun[4])(double, char);
	double tab_rc[4];
	int ntab;

	/* stochastic dynamics: the device holds pv, pa, prevf, randn and ldiff
	 * once ext_on is set; seed keys the random streams, ncall counts the
	 * calls of each stream (DPD, Fokker-Planck, GJF) */
	int ext_on;
	unsigned long long seed;
	unsigned ncall[4];

	/* molecular pressure tensor: sep_init_mol's tables (first atom, chain
	 * length, atom lists as CSR, masses) for the device, the molecular
	 * virial of the pair passes since the last sep_reset_force_mol */
	int mv_on, mv_uploaded, mv_nmol;
	sepmolinfo *mv_info;
	int *mv_first, *mv_nuau, *mv_start, *mv_atoms;
	double *mv_mass;
	double molW[9], molN[9];
	/* molecule tables of sep_berendsen_mol's molecule array on the device */
	sepdev_moltab *bm_tab;
	const sepmol *bm_mols;
	int bm_nmol;

	/* statistics */
	long nbuild;
} rt_ctx;

#define RT_SEED_DEFAULT 0x5eb15eedULL
enum { RT_STREAM_DPD = 1, RT_STREAM_FP = 2, RT_STREAM_GJF = 3 };

rt_ctx *rt_find(const seppart *ptr);
rt_ctx *rt_get(seppart *ptr, const char *caller);   /* exits with sep_error if unknown */
rt_ctx *rt_register(seppart *ptr, long n);
void rt_unregister(seppart *ptr);

/* state transitions */
void rt_need_device(rt_ctx *c, const sepsys *sys);   /* create + upload when needed */
void rt_need_host(rt_ctx *c);                        /* flush + download when needed */
void rt_host_modified(rt_ctx *c);                    /* host data changed: device stale */

/* deferred work and slots */
int rt_new_slot(rt_ctx *c);
void rt_add_op(rt_ctx *c, sepret *ret, int kind, int slot, int chan);
void rt_launch_pass(rt_ctx *c);          /* launch the pending pair pass (force only) */
void rt_open_pass(rt_ctx *c, sepret *ret); /* new pending pass: slots and their operations */
void rt_pass_mol_slot(rt_ctx *c);          /* before launching the pending pass */
void rt_queue_bonded(rt_ctx *c, const sepdev_bterm *t); /* defer a bonded term */
void rt_launch_bonded(rt_ctx *c);        /* launch the pending bonded terms (one kernel) */
void rt_materialize_forces(rt_ctx *c);   /* pending pass + friction + zeroing into stored forces */
void rt_read_slots(rt_ctx *c, sepsys *sys, int leapfrog_slot);   /* sync, apply ops */
/* the same after a deferred fused step: 1 (nothing applied, slots kept)
 * when the step found its list overflowed and must run again */
int rt_read_step_slots(rt_ctx *c, sepsys *sys, int leapfrog_slot);
int rt_ret_pending(rt_ctx *c, const sepret *ret);
void rt_flush(rt_ctx *c);                /* everything pending, then read slots */

/* list management for a pair-force call */
void rt_prepare_list(rt_ctx *c, sepsys *sys, unsigned opt, int brute_excl_bonds);

void rt_check(int rc, const char *what);
void rt_need_ext(rt_ctx *c, const sepsys *sys);    /* stochastic fields on the device */
int rt_type_id(rt_ctx *c, char t);                 /* -1 when no particle has type t */
rt_ctx *rt_find_molinfo(const sepmolinfo *m);      /* context of sep_init_mol's system */
void rt_mv_drop(rt_ctx *c);                        /* forget the molecule tables */
void rt_pairset(rt_ctx *c, sepdev_pairset *ps);   /* pending terms -> device table */   /* sep_error on a device failure */

extern char rt_errbuf[512];

#endif
