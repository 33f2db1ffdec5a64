// dev_pair.cuh - argument block of the pair / step kernels (shared with the graph runner).
#pragma once
#include "dev_common.cuh"
#include "dev_decide.cuh"

// A cubic box measured in fixed-point units u = L / 2^32: u and u^2 as float
// pairs (hi + lo), sigma^2 / u^2 as a float pair and rc^2 / u^2, all rounded
// once from FP64.  Pair terms computed in these units carry no systematic
// error from a rounded scale: s^2 = (s2h + s2l) / r^2 and the rescaled
// force and virial use both halves of u and u^2.
struct LjScale {
	float uh, ul, u2h, u2l, s2h, s2l, rc2s;
};

static inline LjScale lj_scale(double L, double sig2, double rc2)
{
	LjScale c;
	const double u = L / 4294967296.0, u2 = u * u, s2 = sig2 / u2;
	c.uh = (float)u; c.ul = (float)(u - (double)c.uh);
	c.u2h = (float)u2; c.u2l = (float)(u2 - (double)c.u2h);
	c.s2h = (float)s2; c.s2l = (float)(s2 - (double)c.s2h);
	c.rc2s = (float)(rc2 / u2);
	return c;
}

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
	float ushl;                 // ushift - (float)ushift: the shift's remainder
	LjScale sc;                 // cubic boxes: the fixed-point unit and scaled constants
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
	TakeArgs take;             // C-API step: the sums handed to the host at its end
	int skip_obs;              // fused step whose energy and virial nobody reads
	// molecular virial (k_pair<..., MOLV>): molecule of each slot, centres of
	// mass of this pass, per-atom intermolecular force (user order)
	const int *mol;
	const int *gid;
	const int4 *mcm;
	float4 *finter;
	int mslot;
};


// copy a pair set to the device (skipped when the device copy is current)
int sepdev_upload_pairset(sepdev *d, const sepdev_pairset *ps);

void sepdev_fill_args(sepdev *d, PairArgs &a, const sepdev_pairset *ps, double dt, int nh,
		      double alpha, int accumulate, int pslot, int lslot, int parity);
int sepdev_launch_pair(sepdev *d, const sepdev_pairset *ps, PairArgs &a, bool fused);
// centres of mass of the molecules at positions pos (dev_molp.cu)
int sepdev_molvir_cm(sepdev *d, const int4 *pos);
