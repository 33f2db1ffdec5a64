/*
 * sepsampler.h - time-correlation samplers (GB300 implementation).
 *
 * The API and the sampler structure follow the reference's
 * include/sepsampler.h:214-299; programs keep a sepsampler by value and pass
 * its address, so the member list and order are the reference's (the
 * per-sampler structures behind the pointers are this library's own and
 * opaque to programs).  Supported samplers: "sacf" (stress autocorrelation),
 * "vacf" (velocity autocorrelation), "msd" (mean square displacement,
 * non-Gaussian parameter, self-intermediate scattering function), and the
 * molecular "msacf" (molecular stress autocorrelation), "mvacf" (centre-of-
 * mass velocity autocorrelation) and "mgh" (molecular generalised
 * hydrodynamics: momentum, density, energy, spin and dipole correlations
 * per wavevector along y), "gh" (the atomic counterpart: density,
 * momentum and energy correlations along y), "profs" (density, momentum and temperature
 * profiles of one type along z) and "radial" (pair distances histogrammed
 * per type combination), "mmsd" (molecular mean square displacement) and
 * "scatt" (partial coherent scattering functions per type pair), and
 * "mprofs" (molecular density, momentum, temperature, spin and inertia
 * profiles along z) and "mavacf" (the reference's molecular end-to-end
 * dipole-like quantity, autocorrelated).  They write the reference's files (sacf.dat,
 * vacf.dat, msd.dat, msd-gaussparam.dat, msd-incoherent.dat, msd-k.dat,
 * msacf.dat, mvacf.dat, gh-*.dat, mgh-*.dat, profs.dat, radial.dat,
 * radial_info.dat, mmsd*.dat, scatt-*.dat, mprofs.dat) in the same
 * formats.  The particle data
 * a sample needs stays on the GPU: vacf and mvacf keep their window of
 * velocities in device memory, msd and mgh reduce on the device, so sampling
 * costs no download of the particle arrays.  Unlike the reference, mgh does
 * not write the centres of mass, spins and dipoles it evaluates back into
 * the program's molecule array.  Any other sampler name ends the program
 * with sep_error.
 */
#ifndef SEP_GB300_SEPSAMPLER_H
#define SEP_GB300_SEPSAMPLER_H

#include "sepstrct.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sepsacf sepsacf;
typedef struct sepvacf sepvacf;
typedef struct sepgh sepgh;
typedef struct sepprofs sepprofs;
typedef struct sepradial sepradial;
typedef struct sepmsd sepmsd;
typedef struct sepscatt sepscatt;
typedef struct sepmsacf sepmsacf;
typedef struct sepmcacf sepmcacf;
typedef struct sepmgh sepmgh;
typedef struct sepmprofs sepmprofs;
typedef struct sepmvacf sepmvacf;
typedef struct sepmavacf sepmavacf;
typedef struct sepmmsd sepmmsd;

/* Reference include/sepsampler.h:214-239. */
typedef struct {
	sepmol *molptr;

	/* atomic samplers */
	int flag_sacf; sepsacf *sacf;
	int flag_vacf; sepvacf *vacf;
	int flag_gh; sepgh *gh;
	int flag_profs; sepprofs *profs;
	int flag_radial; sepradial *radial;
	int flag_msd; sepmsd *msd;
	int flag_scatt; sepscatt **scatt;

	/* molecular samplers */
	int flag_msacf; sepmsacf *msacf;
	int flag_mcacf; sepmcacf *mcacf;
	int flag_mgh; sepmgh *mgh;
	int flag_mprofs; sepmprofs *mprofs;
	int flag_mvacf; sepmvacf *mvacf;
	int flag_mavacf; sepmavacf *mavacf;
	int flag_mmsd; sepmmsd *mmsd;

	long unsigned msd_counter;
} sepsampler;

/* Reference include/sepsampler.h:247. */
sepsampler sep_init_sampler(void);

/* Reference include/sepsampler.h:275: "sacf", "vacf", "msacf", "mvacf",
 * "mavacf":
 * lvec samples over a time span (double); "gh": lvec samples over a time
 * span (double), number of wave vectors (int); "msd": lvec samples (0:
 * log-spaced) over a time span (double), number of wave vectors (int),
 * particle type (char); "mgh": lvec samples over a time span (double),
 * number of wave vectors (int), safe (int; 0 also evaluates the angular
 * velocities); "profs": lvec bins, particle type (char), sampling interval
 * in steps (int); "radial": lvec bins, sampling interval in steps (int),
 * the types (char *, 1 to 7); "mmsd": as "msd", over the molecules of a
 * molecule type; "scatt": lvec samples, the types (char *, 1 to 7), number
 * of wave vectors (int), time span (double); "mprofs": as "profs", over
 * the molecules of a molecule type.  The molecular samplers need sep_add_mol_sampler first. */
void sep_add_sampler(sepsampler *sptr, const char *sampler, sepsys sys, int lvec, ...);

/* Reference include/sepsampler.h:281. */
void sep_close_sampler(sepsampler *ptr);

/* Reference include/sepsampler.h:291: call once per step n. */
void sep_sample(seppart *pptr, sepsampler *sptr, sepret *ret, sepsys sys, unsigned n);

/* Reference include/sepsampler.h:299: the molecules of msacf, mvacf and mgh. */
void sep_add_mol_sampler(sepsampler *sptr, sepmol *mols);

/* Reference include/sepsampler.h:383: the scatt sampler takes its first type
 * from molecules of even index and its second from molecules of odd index
 * (or none) instead of all particles. */
void sep_set_inter_scatt(sepsampler *sampler);

#ifdef __cplusplus
}
#endif
#endif
