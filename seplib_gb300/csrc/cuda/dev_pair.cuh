// dev_pair.cuh - argument block of the pair / step kernels (shared with the graph runner).
#pragma once
#include "dev_common.cuh"
#include "dev_decide.cuh"

struct PairArgs {
	const int4 *pos;
	int4 *pos_out;
	uint4 *xlo;
	float4 *vhi, *vlo, *frc;
	const int4 *xn;
	int4 *cross;
	const int *nl, *ncnt;
	int maxnb;
	const float *charge;
	float fs[3];
	const sepdev_pairset *ps;
	// single-potential fast path
	float rc2, eps48, eps4, sig2, aw, awh, ushift;
	// tables
	const float2 *tab[SEPDEV_MAXTAB];
	float tab_r2min[SEPDEV_MAXTAB], tab_idr2[SEPDEV_MAXTAB];
	int tab_n[SEPDEV_MAXTAB];
	// integration
	float dt, dt_lo;            // dt as float plus its rounding remainder
	float shi[3], slo[3];
	float alpha;
	const double *alpha_dev;   // when set, alpha is read from device memory
	int nh, accumulate;
	long long *slots;
	int pslot, lslot;
	const unsigned *flags;
	DecideArgs dec;            // graph loop: decision at the end of a fused step
	int skip_obs;              // fused step whose energy and virial nobody reads
	// molecular virial (k_pair<..., MOLV>): molecule of each slot, centres of
	// mass of this pass, per-atom intermolecular force (user order)
	const int *mol;
	const int *gid;
	const int4 *mcm;
	float4 *finter;
	int mslot;
};


void sepdev_fill_args(sepdev *d, PairArgs &a, const sepdev_pairset *ps, double dt, int nh,
		      double alpha, int accumulate, int pslot, int lslot, int parity);
int sepdev_launch_pair(sepdev *d, const sepdev_pairset *ps, PairArgs &a, bool fused);
// centres of mass of the molecules at positions pos (dev_molp.cu)
int sepdev_molvir_cm(sepdev *d, const int4 *pos);
