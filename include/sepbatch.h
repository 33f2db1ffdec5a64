/*
 * sepbatch.h - many independent Lennard-Jones systems stepped together.
 *
 * No counterpart in the reference library: it is an addition of this
 * library.  Each system runs the prgs loop of seplib - sep_force_lj (or
 * sep_force_pairs with sep_lj_shift), sep_nosehoover, sep_leapfrog - with its
 * own box, state, thermostat and neighbour-list updates, exactly as a
 * single-system run through sep_gpu_run would.  On the GPU all systems share
 * one set of arrays and one CUDA graph: small systems (a few hundred
 * particles) cannot fill a GB300 one at a time.
 */
#ifndef SEP_GB300_SEPBATCH_H
#define SEP_GB300_SEPBATCH_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sepb sepb;

/* Results of a system after the last step of the last sepb_run. */
typedef struct {
	double epot, ekin;        /* as sepret.epot, sepret.ekin */
	double pot_P[3][3];       /* as sepret.pot_P */
	double kin_P[3][3];       /* as sepret.kin_P */
	double alpha;             /* Nose-Hoover state, as sep_nosehoover leaves it */
	double max_dist2;         /* as sepsys.max_dist2 */
	double sumv2;             /* sum m v^2 after the last step */
	unsigned nupdate;         /* as sepsys.nupdate_neighb since sepb_set_state */
} sepb_result;

/*
 * nsys systems of npart[s] particles in cubic boxes of edge L[s]; pair cut-off
 * and list cut-off rc (as sepsys.cf) and skin, time step dt.  ljparam =
 * {cf, eps, sigma, aw} as sep_force_lj, or NULL for sep_lj_shift.  Returns
 * NULL on error (message in sep_gpu_error()).
 */
sepb *sepb_create(int nsys, const int *npart, const double *L, double rc, double skin, double dt,
		  const double *ljparam);

/*
 * A batch of mixtures: ntypes (at most 4) particle types with one
 * Lennard-Jones parameter set {cf, eps, sigma, aw} per type pair, as one
 * sep_force_lj(ptr, "ab", param_ab, ...) call per pair of types would give
 * (the energies of the calls add).  ljparams holds ntypes x ntypes sets of
 * four doubles, set [a][b] equal to set [b][a]; eps = 0 leaves a type pair
 * without a term.  The list cut-off is the largest cf plus skin.  Types are
 * set per system with sepb_set_types (all type 0 otherwise).
 */
sepb *sepb_create_typed(int nsys, const int *npart, const double *L, double skin, double dt,
			int ntypes, const double *ljparams);

/* Type ids (0 .. ntypes-1) of the n particles of system s of a typed batch;
 * call it after sepb_set_state of that system and before the next run. */
int sepb_set_types(sepb *b, int s, const int *type);

/* Positions (3 n, wrapped into the box), velocities (3 n) and masses (n, or
 * NULL for 1) of system s.  A system set here starts afresh: its first step
 * reports a list update, as the first sep_leapfrog of a program does. */
int sepb_set_state(sepb *b, int s, const double *x, const double *v, const double *m);

/* Nose-Hoover on every system: targets T0[s], tau as the fourth argument of
 * sep_nosehoover, alpha[s] initial states (NULL: 0).  T0 == NULL: NVE. */
int sepb_set_thermostat(sepb *b, const double *T0, double tau, const double *alpha);

/* nsteps of every system. */
int sepb_run(sepb *b, long nsteps);

/* Timing helper: the same steps launched one at a time, each bracketed by
 * CUDA events, with flush_bytes written before each step outside the spans
 * so no step finds the previous one's data in L2; *ms_steps = the summed
 * spans. */
int sepb_run_timed(sepb *b, long nsteps, long flush_bytes, double *ms_steps);

/* Positions, velocities and forces of system s (any may be NULL). */
int sepb_get_state(sepb *b, int s, double *x, double *v, double *f);

/* nsys results. */
int sepb_get_results(sepb *b, sepb_result *out);

/* Device slots in use (particles plus the padding that aligns systems to warps). */
long sepb_particles(const sepb *b);

void sepb_destroy(sepb *b);

#ifdef __cplusplus
}
#endif
#endif
