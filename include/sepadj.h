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

/* Initial positions (3 n), velocities (3 n) and masses (n or NULL) of replica r. */
int sepadj_set_state(sepadj *a, int r, const double *x, const double *v, const double *m);

/* nsteps NVE steps of every replica from the initial states; loss[r]. */
int sepadj_forward(sepadj *a, long nsteps, double *loss);

/* Gradients of the last forward's losses: dloss_deps[r], dloss_dsigma[r]
 * and dloss_dx0 (3 n of replica 0, then replica 1, ...; may be NULL). */
int sepadj_backward(sepadj *a, double *dloss_deps, double *dloss_dsigma, double *dloss_dx0);

void sepadj_destroy(sepadj *a);

#ifdef __cplusplus
}
#endif
#endif
