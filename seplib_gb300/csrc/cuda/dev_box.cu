// dev_box.cu - box changes on the device: compression and the Berendsen
// barostat (reference source/sepmisc.c:892-1084).
//
// The reference multiplies the box edges and, separately, each position
// coordinate by a factor, and leaves xn (the positions of the last list
// update) as they are.  Positions here are fractions of the box, so every
// coordinate is rebuilt from its FP64 value times the factor and
// re-expressed in the new box, in FP64 as the reference computes it.  A
// coordinate the scaling carries past the edge is wrapped and counted as a
// crossing, which the reference does at its next integrator step.  xn keeps
// its absolute value in the new box, so the skin test sees the displacement
// the reference's sees.
#include <math.h>
#include "dev_common.cuh"

struct Rescale {
	double L0[3], L1[3], sx[3];
};

__global__ void k_rescale(long n, int4 *pos, uint4 *xlo, int4 *xn, int4 *cross, Rescale r)
{
	const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
	if (i >= n) return;
	const int4 p = pos[i];
	const uint4 lo = xlo[i];
	const int4 q = xn[i];
	const unsigned ph[3] = {(unsigned)p.x, (unsigned)p.y, (unsigned)p.z};
	const unsigned pl[3] = {lo.x, lo.y, lo.z};
	const unsigned qh[3] = {(unsigned)q.x, (unsigned)q.y, (unsigned)q.z};
	unsigned h[3], l[3], hn[3], ln;
	int cr[3];
#pragma unroll
	for (int k = 0; k < 3; k++) {
		double x = __dmul_rn(from_fixed_dev(ph[k], pl[k], r.L0[k]), r.sx[k]);
		cr[k] = 0;
		if (x >= r.L1[k]) { x = __dsub_rn(x, r.L1[k]); cr[k] = 1; }
		to_fixed_dev(x, r.L1[k], h[k], l[k]);
		to_fixed_dev(from_fixed_dev(qh[k], 0u, r.L0[k]), r.L1[k], hn[k], ln);
	}
	pos[i] = make_int4((int)h[0], (int)h[1], (int)h[2], p.w);
	xlo[i] = make_uint4(l[0], l[1], l[2], 0u);
	xn[i] = make_int4((int)hn[0], (int)hn[1], (int)hn[2], q.w);
	if (cr[0] | cr[1] | cr[2]) {
		int4 c = cross[i];
		c.x += cr[0]; c.y += cr[1]; c.z += cr[2];
		cross[i] = c;
	}
}

extern void sepdev_runner_free(sepdev *d);

extern "C" int sepdev_rescale_box(sepdev *d, const double *L1, const double *sx)
{
	Rescale r;
	for (int k = 0; k < 3; k++) {
		if (!(L1[k] > 0.0) || !(sx[k] > 0.0)) return SEPDEV_EINVAL;
		r.L0[k] = d->L[k];
		r.L1[k] = L1[k];
		r.sx[k] = sx[k];
	}
	k_rescale<<<grid_for(d->n, 256), 256, 0, d->st>>>(d->n, d->pos[d->cur], d->xlo, d->xn, d->cross, r);
	CKL(d);
	for (int k = 0; k < 3; k++) {
		d->L[k] = L1[k];
		d->fscale[k] = (float)(L1[k] / 4294967296.0);
	}
	// captured loop graphs hold the old box's scale factors
	sepdev_runner_free(d);
	return SEPDEV_OK;
}
