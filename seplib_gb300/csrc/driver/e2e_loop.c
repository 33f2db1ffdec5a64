/*
 * e2e_loop.c - the prgs-style MD step loop through the sep C API, timed by
 * wall clock the way a seplib program runs it: prgs/prg0.c's loop with a
 * Nose-Hoover thermostat,
 *
 *     sep_reset_retval; sep_reset_force; sep_force_pairs(lj_shift);
 *     sep_nosehoover; sep_leapfrog
 *
 * or, with a topology, the molecular step of prgs/prg2.c (LJ between
 * different molecules, harmonic bonds and angles, Ryckaert-Bellemans
 * torsions, Nose-Hoover, leap-frog) with the united-atom butane force field
 * (bonds k = 33615, l0 = 0.4; angles k = 866, theta0 = 1.9; torsion
 * coefficients 15.5, 20.3, -21.9, -5.1, 43.8, -52.6).
 *
 * The particle arrays live in host memory.  The first timed step uploads
 * them (the state is marked host-modified before it); every step reads its
 * sepret values back; the final sep_gpu_sync (timed) downloads x, v and f.
 *
 *   sep_e2e_loop STATE STEPS WARMUP FLUSH_BYTES RC DT SKIN T0 TAU [TOPOLOGY]
 *                [--tune NCLASS (NMAX TEAM GROUPS CELLF) x NCLASS]
 *
 * --tune applies a table of kernel parameters by system size
 * (sep_gpu_set_tuning) before the run, as the autotuner chose it.
 *
 * STATE is a binary file: int64 n, double L[3], double x[3n], double v[3n],
 * double m[n], char type[n].  Before every timed step FLUSH_BYTES are
 * written on the device (untimed) so no step finds the previous one's data
 * in L2.  Prints one JSON line.
 */
#define _POSIX_C_SOURCE 199309L
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "sep.h"

static double now(void)
{
	struct timespec t;
	clock_gettime(CLOCK_MONOTONIC, &t);
	return t.tv_sec + 1e-9 * t.tv_nsec;
}

int main(int argc, char **argv)
{
	for (int k = 10; k < argc; k++) {
		if (strcmp(argv[k], "--tune") != 0) continue;
		sep_gpu_tuning t;
		memset(&t, 0, sizeof t);
		t.nclass = k + 1 < argc ? atoi(argv[k + 1]) : 0;
		if (t.nclass < 1 || t.nclass > SEP_GPU_NCLASS || k + 2 + 4 * t.nclass != argc) {
			fprintf(stderr, "bad --tune table\n");
			return 2;
		}
		for (int c = 0; c < t.nclass; c++) {
			t.nmax[c] = atol(argv[k + 2 + 4 * c]);
			t.team[c] = atoi(argv[k + 3 + 4 * c]);
			t.groups[c] = atoi(argv[k + 4 + 4 * c]);
			t.cellf[c] = atof(argv[k + 5 + 4 * c]);
		}
		if (sep_gpu_set_tuning(&t) != 0) {
			fprintf(stderr, "sep_gpu_set_tuning rejected the table\n");
			return 2;
		}
		argc = k;
		break;
	}
	if (argc != 10 && argc != 11) {
		fprintf(stderr, "usage: %s STATE STEPS WARMUP FLUSH_BYTES RC DT SKIN T0 TAU [TOPOLOGY]\n", argv[0]);
		return 2;
	}
	const char *top = argc == 11 ? argv[10] : NULL;
	const long steps = atol(argv[2]), warmup = atol(argv[3]), flush = atol(argv[4]);
	const double rc = atof(argv[5]), dt = atof(argv[6]), skin = atof(argv[7]);
	const double temp = atof(argv[8]), tau = atof(argv[9]);
	FILE *fp = fopen(argv[1], "rb");
	if (!fp) { perror(argv[1]); return 2; }
	int64_t n64;
	double L[3];
	if (fread(&n64, sizeof n64, 1, fp) != 1 || fread(L, sizeof(double), 3, fp) != 3) return 2;
	const long n = (long)n64;
	double *xv = malloc(sizeof(double) * 7 * n);
	char *ty = malloc(n);
	if (!xv || !ty || fread(xv, sizeof(double), 7 * n, fp) != (size_t)(7 * n) ||
	    fread(ty, 1, n, fp) != (size_t)n)
		return 2;
	fclose(fp);

	seppart *atoms = sep_init(n, SEP_NEIGHB);
	for (long i = 0; i < n; i++) {
		for (int k = 0; k < 3; k++) {
			atoms[i].x[k] = xv[3 * i + k];
			atoms[i].v[k] = xv[3 * n + 3 * i + k];
		}
		atoms[i].m = xv[6 * n + i];
		atoms[i].type = ty[i];
	}
	free(xv);
	const char types[3] = {ty[0], ty[0], 0};
	free(ty);
	sepsys sys = sep_sys_setup(L[0], L[1], L[2], rc, dt, n, SEP_LLIST_NEIGHBLIST);
	sep_set_skin(&sys, skin);
	if (top) sep_read_topology_file(atoms, top, &sys, 'q');
	double rb[6] = {15.5, 20.3, -21.9, -5.1, 43.8, -52.6};
	sepret ret;
	double alpha = 0.0;

#define STEP()                                                                              \
	do {                                                                                \
		sep_reset_retval(&ret);                                                     \
		sep_reset_force(atoms, &sys);                                               \
		if (top) {                                                                  \
			sep_force_pairs(atoms, types, rc, sep_lj_shift, &sys, &ret, SEP_EXCL_SAME_MOL); \
			sep_stretch_harmonic(atoms, 0, 0.4, 33615.0, &sys, &ret);          \
			sep_angle_harmonic(atoms, 0, 1.9, 866.0, &sys, &ret);              \
			sep_torsion_Ryckaert(atoms, 0, rb, &sys, &ret);                     \
		} else {                                                                    \
			sep_force_pairs(atoms, types, rc, sep_lj_shift, &sys, &ret, SEP_ALL);      \
		}                                                                           \
		sep_nosehoover(atoms, temp, &alpha, tau, &sys);                             \
		sep_leapfrog(atoms, &sys, &ret);                                            \
	} while (0)

	for (long s = 0; s < warmup; s++) STEP();
	sep_gpu_sync(atoms);
	sep_gpu_invalidate(atoms);          /* the first timed step uploads the host arrays */

	const unsigned u0 = sys.nupdate_neighb;
	double t = 0.0, t_first = 0.0;
	for (long s = 0; s < steps; s++) {
		sep_gpu_flush_l2(atoms, flush);
		const double t0 = now();
		STEP();
		const double dtw = now() - t0;
		t += dtw;
		if (s == 0) t_first = dtw;
	}
	const double t0 = now();
	sep_gpu_sync(atoms);
	const double t_down = now() - t0;
	t += t_down;
	printf("{\"seconds\": %.9f, \"steps\": %ld, \"n\": %ld, \"rebuilds\": %u, \"first_step_s\": %.9f, "
	       "\"final_download_s\": %.9f, \"epot\": %.10g, \"ekin\": %.10g}\n",
	       t, steps, n, sys.nupdate_neighb - u0, t_first, t_down, ret.epot, ret.ekin);
	sep_close(atoms, n);
	sep_free_sys(&sys);
	return 0;
}
