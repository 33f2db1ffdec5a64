/*
 * sepadj.h - gradients of an MD loss through the LJ force and leap-frog
 * (reverse mode, with checkpoints).
 *
 * No counterpart in the reference library: it is an addition of this
 * library.  Each of nrep independent replicas runs the NVE prgs loop
 * (sep_force_lj with param = {cf, eps, sigma, aw}, sep_leapfrog) for nsteps
 * steps; the loss of a replica is the time average
 *
 *     L = (1/K) sum_{n=0}^{K-1} ( epot_n + p_n ),
 *     p_n = ( tr kin_P_n + tr pot_P_n ) / (3 V)
 *
 * of the step's sepret.epot and pressure (sep_pressure_tensor).  The backward
 * pass returns dL/d eps, dL/d sigma and dL/d x0 (initial positions) of every
 * replica.  It differentiates the forces the forward pass uses, that is the
 * reference's LJ force including its sigma^2/r^2 factor
 * (source/sepprfrc.c:743-1000).
 *
 * The forward pass keeps the replica state every ckpt_every steps; the
 * backward pass recomputes each segment from its checkpoint and sweeps it
 * backwards.  Pair terms are FP32 like the forward's; the adjoint state of
 * every particle is accumulated in FP64.
 */
#ifndef SEP_GB300_SEPADJ_H
#define SEP_GB300_SEPADJ_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sepadj sepadj;

/* nrep replicas of npart[r] particles in cubic boxes of edge L[r]; list
 * cut-off rc + skin, time step dt; ljparam = {cf, eps, sigma, aw} (required);
 * a checkpoint every ckpt_every steps.  NULL on error (sep_gpu_error()). */
sepadj *sepadj_create(int nrep, const int *npart, const double *L, double rc, double skin,
		      double dt, const double *ljparam, int ckpt_every);

/*
 * Mixtures: ntypes (at most 4) particle types with one parameter set
 * {cf, eps, sigma, aw} per type pair, the loop being one sep_force_lj call
 * per pair of types ("ab", param_ab; the energies add) and sep_leapfrog.
 * ljparams holds ntypes x ntypes sets of four doubles, set [a][b] equal to
 * set [b][a]; eps = 0 leaves a type pair without a term.  The list cut-off
 * is the largest cf plus skin.  Gradients come from sepadj_backward_typed.
 */
sepadj *sepadj_create_typed(int nrep, const int *npart, const double *L, double skin, double dt,
			    int ntypes, const double *ljparams, int ckpt_every);

/* Initial positions (3 n), velocities (3 n) and masses (n or NULL) of replica r. */
int sepadj_set_state(sepadj *a, int r, const double *x, const double *v, const double *m);

/* Type ids (0 .. ntypes-1) of the particles of replica r (typed adjoint);
 * after sepadj_set_state of that replica. */
int sepadj_set_types(sepadj *a, int r, const int *type);

/* nsteps NVE steps of every replica from the initial states; loss[r]. */
int sepadj_forward(sepadj *a, long nsteps, double *loss);

/* Gradients of the last forward's losses: dloss_deps[r], dloss_dsigma[r]
 * and dloss_dx0 (3 n of replica 0, then replica 1, ...; may be NULL). */
int sepadj_backward(sepadj *a, double *dloss_deps, double *dloss_dsigma, double *dloss_dx0);

/* The same for a typed adjoint: dloss_deps and dloss_dsigma hold
 * nrep x ntypes x ntypes values, [r][a][b] = [r][b][a] the gradient with
 * respect to the one eps (sigma) of type pair {a, b}. */
int sepadj_backward_typed(sepadj *a, double *dloss_deps, double *dloss_dsigma, double *dloss_dx0);

/* Positions and velocities (3 n each, either may be NULL) of replica r at
 * the end of the last forward pass; call it before sepadj_backward, whose
 * recomputation leaves other states on the device. */
int sepadj_get_state(sepadj *a, int r, double *x, double *v);

void sepadj_destroy(sepadj *a);

#ifdef __cplusplus
}
#endif
#endif
