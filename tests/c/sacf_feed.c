/*
 * Feeds a stress-autocorrelation sampler with synthetic sepret values (no
 * particles, no GPU): step n sets pot_P to a known tensor and calls
 * sep_sample; the test recomputes sacf.dat from the same values.
 *
 *   usage: sacf_feed <nsteps>
 */
#include <stdlib.h>
#include "sep.h"

int main(int argc, char **argv)
{
	const int nsteps = argc > 1 ? atoi(argv[1]) : 400;
	const double L = 10.0;
	sepsys sys;
	memset(&sys, 0, sizeof sys);
	sys.length[0] = sys.length[1] = sys.length[2] = L;
	sys.volume = L * L * L;
	sys.dt = 0.005;
	sys.npart = 100;
	sepsampler s = sep_init_sampler();
	sep_add_sampler(&s, "sacf", sys, 20, 0.8);   /* 20 samples, every 8 steps */
	sepret ret;
	for (int n = 0; n < nsteps; n++) {
		memset(&ret, 0, sizeof ret);
		for (int k = 0; k < 3; k++)
			for (int kk = 0; kk < 3; kk++)
				ret.pot_P[k][kk] = sin(0.37 * n + k + 2.0 * kk) * (1.0 + 0.1 * k * kk);
		ret.kin_P[0][1] = ret.kin_P[1][0] = 0.25 * cos(0.11 * n);
		sep_sample(NULL, &s, &ret, sys, n);
	}
	sep_close_sampler(&s);
	return 0;
}
