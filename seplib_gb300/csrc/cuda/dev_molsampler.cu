// dev_molsampler.cu - device parts of the molecular samplers mvacf and mgh,
// and the molecular Berendsen barostat.
//
// The reference (source/sepsampler.c:1231-1410 mgh, :1757-1816 mvacf)
// downloads nothing itself but walks every molecule on the host at each
// sample: centre of mass (source/sepmol.c:683-729), centre-of-mass velocity
// (:731-748), spin angular momentum and inertia tensor (:750-825) and the
// charge dipole (:1036-1083), then per wavevector sums over the molecules.
// Here one thread per molecule forms these from the device state, a second
// kernel sums them per wavevector with a fixed reduction order, and only
// nk x 18 numbers come back per sample.  mvacf keeps the molecular
// x-velocities of a block in a device ring (the vacf ring of dev_sampler.cu
// sized by the molecule count).
//
// Positions are taken from the full 64-bit fixed-point words, as fractions
// of the box in FP64; all molecular quantities are FP64.
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include "dev_common.cuh"

#define MSB 128

struct sepdev_moltab {
	int nmol, nblk;
	int *first, *nuau, *start, *atoms;
	double *mass;
	double *props;     // [nmol][MP_N]
	double *pel;       // [nmol][3] last dipole (kept when a molecule has no +/- charges)
	double *kvec;      // [nk]
	int nk_alloc;
	double *part;      // [nk][nblk][MG_N]
	double *sum;       // [nk * MG_N]
};

enum { MP_Y, MP_M, MP_MVX, MP_MVY, MP_EK, MP_SZ, MP_SY, MP_PY, MP_WX, MP_N };
#define MG_N 18

__device__ __forceinline__ double frac64(int hi, unsigned lo)
{
	return ldexp((double)(((unsigned long long)(unsigned)hi << 32) | lo), -64);
}

__device__ __forceinline__ double wrap_half(double f)
{
	if (f > 0.5) return f - 1.0;
	if (f < -0.5) return f + 1.0;
	return f;
}

struct MolArgs {
	int nmol;
	const int *first, *nuau, *start, *atoms, *inv;
	const double *mass;
	const int4 *pos;
	const uint4 *xlo;
	const float4 *vhi, *vlo;
	const float *charge;
	double L[3];
	int unsafe;
	double *props, *pel;
};

// per molecule: the centre of mass (chain of consecutive user indices from
// the first atom, bonds unwrapped by the minimum image, wrapped into the
// box), velocity, kinetic energy M v^2 / 2, spin s = sum dcm x m v about the
// centre of mass, the charge dipole and, in the unsafe mode, the angular
// velocity I^-1 s
__global__ void __launch_bounds__(MSB) k_mol_props(MolArgs a)
{
	const int m = blockIdx.x * MSB + threadIdx.x;
	if (m >= a.nmol) return;
	const int a0 = a.first[m];
	double cmf[3];
	{
		const int s0 = a.inv[a0];
		const int4 p0 = a.pos[s0];
		const uint4 l0 = a.xlo[s0];
		unsigned long long prev[3] = {((unsigned long long)(unsigned)p0.x << 32) | l0.x,
					      ((unsigned long long)(unsigned)p0.y << 32) | l0.y,
					      ((unsigned long long)(unsigned)p0.z << 32) | l0.z};
		const double f0[3] = {ldexp((double)prev[0], -64), ldexp((double)prev[1], -64),
				      ldexp((double)prev[2], -64)};
		double off[3] = {0.0, 0.0, 0.0}, acc[3] = {0.0, 0.0, 0.0};
		for (int q = 0; q < a.nuau[m]; q++) {
			const int s = a.inv[a0 + q];
			const int4 p = a.pos[s];
			const uint4 l = a.xlo[s];
			const unsigned long long X[3] = {((unsigned long long)(unsigned)p.x << 32) | l.x,
							 ((unsigned long long)(unsigned)p.y << 32) | l.y,
							 ((unsigned long long)(unsigned)p.z << 32) | l.z};
			const double ma = (double)a.vhi[s].w;
			for (int k = 0; k < 3; k++) {
				if (q > 0) off[k] += ldexp((double)(long long)(X[k] - prev[k]), -64);
				prev[k] = X[k];
				acc[k] += ma * off[k];
			}
		}
		const double M = a.mass[m];
		for (int k = 0; k < 3; k++) {
			double f = f0[k] + acc[k] / M;
			if (f >= 1.0) f -= 1.0;
			else if (f < 0.0) f += 1.0;
			cmf[k] = f;
		}
	}
	const double M = a.mass[m];
	double v[3] = {0.0, 0.0, 0.0}, s[3] = {0.0, 0.0, 0.0};
	double I00 = 0.0, I11 = 0.0, I22 = 0.0, I01 = 0.0, I02 = 0.0, I12 = 0.0;
	double rpos[3] = {0.0, 0.0, 0.0}, rneg[3] = {0.0, 0.0, 0.0}, sumz = 0.0;
	int npos = 0, nneg = 0;
	for (int q = a.start[m]; q < a.start[m + 1]; q++) {
		const int sl = a.inv[a.atoms[q]];
		const int4 p = a.pos[sl];
		const uint4 l = a.xlo[sl];
		const float4 vh = a.vhi[sl], vl = a.vlo[sl];
		const double ma = (double)vh.w;
		const double va[3] = {(double)vh.x + (double)vl.x, (double)vh.y + (double)vl.y,
				      (double)vh.z + (double)vl.z};
		const double fx[3] = {frac64(p.x, l.x), frac64(p.y, l.y), frac64(p.z, l.z)};
		double d[3], pm[3];
		for (int k = 0; k < 3; k++) {
			v[k] += va[k] * ma;
			d[k] = wrap_half(fx[k] - cmf[k]) * a.L[k];
			pm[k] = va[k] * ma;
		}
		s[0] += d[1] * pm[2] - d[2] * pm[1];
		s[1] += d[2] * pm[0] - d[0] * pm[2];
		s[2] += d[0] * pm[1] - d[1] * pm[0];
		I00 += ma * (d[1] * d[1] + d[2] * d[2]);
		I11 += ma * (d[0] * d[0] + d[2] * d[2]);
		I22 += ma * (d[0] * d[0] + d[1] * d[1]);
		I01 -= ma * d[0] * d[1];
		I02 -= ma * d[0] * d[2];
		I12 -= ma * d[1] * d[2];
		if (a.charge) {
			const double z = (double)a.charge[sl];
			if (z > 0.0) {
				for (int k = 0; k < 3; k++) rpos[k] += cmf[k] * a.L[k] + d[k];
				sumz += z;
				npos++;
			} else if (z < 0.0) {
				for (int k = 0; k < 3; k++) rneg[k] += cmf[k] * a.L[k] + d[k];
				nneg++;
			}
		}
	}
	for (int k = 0; k < 3; k++) v[k] /= M;
	if (npos > 0 && nneg > 0)
		for (int k = 0; k < 3; k++) a.pel[3 * m + k] = sumz * (rpos[k] / npos - rneg[k] / nneg);
	double ek = 0.0;
	for (int k = 0; k < 3; k++) ek += 0.5 * M * v[k] * v[k];
	double wx = 0.0;
	if (a.unsafe) {
		// I w = s; a singular tensor (a linear molecule) takes the mean
		// principal moment, trace / 3
		const double det = I00 * (I11 * I22 - I12 * I12) - I01 * (I01 * I22 - I12 * I02) +
				   I02 * (I01 * I12 - I11 * I02);
		if (fabs(det) < DBL_EPSILON)
			wx = s[0] / ((I00 + I11 + I22) / 3.0);
		else
			wx = (s[0] * (I11 * I22 - I12 * I12) - I01 * (s[1] * I22 - I12 * s[2]) +
			      I02 * (s[1] * I12 - I11 * s[2])) / det;
	}
	double *o = a.props + (long)m * MP_N;
	o[MP_Y] = cmf[1] * a.L[1];
	o[MP_M] = M;
	o[MP_MVX] = M * v[0];
	o[MP_MVY] = M * v[1];
	o[MP_EK] = ek;
	o[MP_SZ] = s[2];
	o[MP_SY] = s[1];
	o[MP_PY] = a.pel[3 * m + 1];
	o[MP_WX] = wx;
}

// blockIdx.y = wavevector j: per block the sums over its molecules of
// e^{i k_j y} times M, M vx, M vy, the kinetic energy, 1, s_z, s_y, the
// dipole's y component and w_x (re, im interleaved)
__global__ void __launch_bounds__(MSB) k_mgh_sums(int nmol, const double *props, const double *kvec,
						  double *part)
{
	__shared__ double red[MSB / 32][MG_N];
	const int m = blockIdx.x * MSB + threadIdx.x;
	const int j = blockIdx.y;
	double t[MG_N];
	for (int q = 0; q < MG_N; q++) t[q] = 0.0;
	if (m < nmol) {
		const double *o = props + (long)m * MP_N;
		double sn, cs;
		sincos(kvec[j] * o[MP_Y], &sn, &cs);
		const double w[9] = {o[MP_M], o[MP_MVX], o[MP_MVY], o[MP_EK], 1.0, o[MP_SZ], o[MP_SY], o[MP_PY],
				     o[MP_WX]};
		for (int q = 0; q < 9; q++) {
			t[2 * q] = w[q] * cs;
			t[2 * q + 1] = w[q] * sn;
		}
	}
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	for (int q = 0; q < MG_N; q++) {
		double x = t[q];
		for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
		if (lane == 0) red[wid][q] = x;
	}
	__syncthreads();
	if (threadIdx.x < MG_N) {
		double x = 0.0;
		for (int w = 0; w < MSB / 32; w++) x += red[w][threadIdx.x];
		part[((long)j * gridDim.x + blockIdx.x) * MG_N + threadIdx.x] = x;
	}
}

// one thread per (j, q): the blocks' partial sums in order; row nk * MG_N
// (an extra thread) sums the kinetic energies
__global__ void k_mgh_rows(int nk, int nblk, int nmol, const double *part, const double *props, double *out)
{
	const int r = blockIdx.x * blockDim.x + threadIdx.x;
	if (r < nk * MG_N) {
		const int j = r / MG_N, q = r % MG_N;
		double s = 0.0;
		for (int b = 0; b < nblk; b++) s += part[((long)j * nblk + b) * MG_N + q];
		out[r] = s;
	} else if (r == nk * MG_N) {
		double s = 0.0;
		for (int m = 0; m < nmol; m++) s += props[(long)m * MP_N + MP_EK];
		out[r] = s;
	}
}

// mvacf: row[m] = x-velocity of molecule m's centre of mass
__global__ void k_mol_vx(int nmol, const int *start, const int *atoms, const int *inv, const float4 *vhi,
			 const float4 *vlo, const double *mass, double *row)
{
	const int m = blockIdx.x * blockDim.x + threadIdx.x;
	if (m >= nmol) return;
	double v = 0.0;
	for (int q = start[m]; q < start[m + 1]; q++) {
		const int s = inv[atoms[q]];
		v += ((double)vhi[s].x + (double)vlo[s].x) * (double)vhi[s].w;
	}
	row[m] = v / mass[m];
}

// ---- host side ---------------------------------------------------------------

extern "C" void sepdev_moltab_destroy(sepdev_moltab *t)
{
	if (!t) return;
	void *b[] = {t->first, t->nuau, t->start, t->atoms, t->mass, t->props, t->pel, t->kvec, t->part, t->sum};
	for (size_t k = 0; k < sizeof b / sizeof b[0]; k++)
		if (b[k]) cudaFree(b[k]);
	free(t);
}

extern "C" int sepdev_moltab_create(sepdev *d, int nmol, const int *first, const int *nuau, const int *start,
				    const int *atoms, const double *mass, sepdev_moltab **out)
{
	*out = NULL;
	if (nmol < 1) return SEPDEV_EINVAL;
	for (int m = 0; m < nmol; m++)
		if (nuau[m] < 1 || first[m] < 0 || first[m] + nuau[m] > d->n || start[m + 1] < start[m])
			return SEPDEV_EINVAL;
	for (int q = 0; q < start[nmol]; q++)
		if (atoms[q] < 0 || atoms[q] >= d->n) return SEPDEV_EINVAL;
	sepdev_moltab *t = (sepdev_moltab *)calloc(1, sizeof *t);
	if (!t) return SEPDEV_ENOMEM;
	t->nmol = nmol;
	t->nblk = (nmol + MSB - 1) / MSB;
	const int na = start[nmol] > 0 ? start[nmol] : 1;
	cudaError_t e = cudaMalloc((void **)&t->first, sizeof(int) * nmol);
	if (e == cudaSuccess) e = cudaMalloc((void **)&t->nuau, sizeof(int) * nmol);
	if (e == cudaSuccess) e = cudaMalloc((void **)&t->start, sizeof(int) * (nmol + 1));
	if (e == cudaSuccess) e = cudaMalloc((void **)&t->atoms, sizeof(int) * na);
	if (e == cudaSuccess) e = cudaMalloc((void **)&t->mass, sizeof(double) * nmol);
	if (e == cudaSuccess) e = cudaMalloc((void **)&t->props, sizeof(double) * MP_N * nmol);
	if (e == cudaSuccess) e = cudaMalloc((void **)&t->pel, sizeof(double) * 3 * nmol);
	if (e == cudaSuccess) e = cudaMemcpy(t->first, first, sizeof(int) * nmol, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(t->nuau, nuau, sizeof(int) * nmol, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(t->start, start, sizeof(int) * (nmol + 1), cudaMemcpyHostToDevice);
	if (e == cudaSuccess && start[nmol] > 0)
		e = cudaMemcpy(t->atoms, atoms, sizeof(int) * start[nmol], cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(t->mass, mass, sizeof(double) * nmol, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemset(t->pel, 0, sizeof(double) * 3 * nmol);
	if (e != cudaSuccess) {
		sepdev_moltab_destroy(t);
		sepdev_set_error("molecule tables", e);
		return SEPDEV_ENOMEM;
	}
	*out = t;
	return SEPDEV_OK;
}

extern "C" int sepdev_mvacf_store(sepdev *d, sepdev_moltab *t, sepdev_vacf *v, int index)
{
	double *row = sepdev_vacf_row(v, index);
	if (!row || sepdev_vacf_count(v) != t->nmol) return SEPDEV_EINVAL;
	k_mol_vx<<<grid_for(t->nmol, 128), 128, 0, d->st>>>(t->nmol, t->start, t->atoms, d->inv, d->vhi, d->vlo,
							   t->mass, row);
	CKL(d);
	return SEPDEV_OK;
}

extern "C" int sepdev_mgh_sample(sepdev *d, sepdev_moltab *t, int nk, const double *k, int unsafe, double *out)
{
	if (nk < 1) return SEPDEV_EINVAL;
	if (nk > t->nk_alloc) {
		cudaFree(t->kvec); cudaFree(t->part); cudaFree(t->sum);
		t->kvec = t->part = t->sum = NULL;
		t->nk_alloc = 0;
		cudaError_t e = cudaMalloc((void **)&t->kvec, sizeof(double) * nk);
		if (e == cudaSuccess) e = cudaMalloc((void **)&t->part, sizeof(double) * MG_N * nk * t->nblk);
		if (e == cudaSuccess) e = cudaMalloc((void **)&t->sum, sizeof(double) * (MG_N * nk + 1));
		if (e != cudaSuccess) { sepdev_set_error("mgh buffers", e); return SEPDEV_ENOMEM; }
		t->nk_alloc = nk;
	}
	CK(cudaMemcpyAsync(t->kvec, k, sizeof(double) * nk, cudaMemcpyHostToDevice, d->st));
	MolArgs a;
	a.nmol = t->nmol;
	a.first = t->first; a.nuau = t->nuau; a.start = t->start; a.atoms = t->atoms; a.inv = d->inv;
	a.mass = t->mass;
	a.pos = d->pos[d->cur]; a.xlo = d->xlo; a.vhi = d->vhi; a.vlo = d->vlo;
	a.charge = d->has_charge ? d->charge : NULL;
	for (int q = 0; q < 3; q++) a.L[q] = d->L[q];
	a.unsafe = unsafe;
	a.props = t->props; a.pel = t->pel;
	k_mol_props<<<t->nblk, MSB, 0, d->st>>>(a);
	k_mgh_sums<<<dim3(t->nblk, nk), MSB, 0, d->st>>>(t->nmol, t->props, t->kvec, t->part);
	k_mgh_rows<<<grid_for(MG_N * nk + 1, 128), 128, 0, d->st>>>(nk, t->nblk, t->nmol, t->part, t->props, t->sum);
	d->launches += 2;
	CKL(d);
	CK(cudaMemcpyAsync(out, t->sum, sizeof(double) * (MG_N * nk + 1), cudaMemcpyDeviceToHost, d->st));
	CK(cudaStreamSynchronize(d->st));
	return SEPDEV_OK;
}

// ---- molecular Berendsen barostat (source/sepmisc.c:948-990) ------------------
//
// The reference takes each molecule's centre of mass (source/sepmol.c:
// 683-729), scales its z coordinate by xi^(1/3) while the box edge L_z is
// scaled by xi, and moves every atom of the molecule with it, keeping its
// offset from the centre of mass; the new z is wrapped once into the new box
// without counting a crossing.  Atoms outside molecules keep their absolute
// z (one beyond the new edge is wrapped and counted, as at the reference's
// next integrator step).  Same FP64 operations as the reference.

__device__ __forceinline__ double coord(const int4 &p, const uint4 &l, int k, double L)
{
	return k == 0 ? from_fixed_dev((unsigned)p.x, l.x, L)
		      : (k == 1 ? from_fixed_dev((unsigned)p.y, l.y, L) : from_fixed_dev((unsigned)p.z, l.z, L));
}

// coordinate k of the centre of mass, in the reference's order: the chain
// of consecutive user indices from the first atom, each step's minimum
// image added to the previous position
__device__ double mol_cm_k(int m, int k, const int *first, const int *nuau, const double *mass, const int4 *pos,
			   const uint4 *xlo, const int *inv, const float4 *vhi, double L)
{
	const int a0 = first[m];
	int s = inv[a0];
	double xprev = coord(pos[s], xlo[s], k, L), chain = xprev;
	double acc = __dmul_rn((double)vhi[s].w, chain);
	for (int q = 1; q < nuau[m]; q++) {
		s = inv[a0 + q];
		const double x = coord(pos[s], xlo[s], k, L);
		double r = __dsub_rn(x, xprev);
		if (r > 0.5 * L) r = __dsub_rn(r, L);
		else if (r < -0.5 * L) r = __dadd_rn(r, L);
		chain = __dadd_rn(chain, r);
		acc = __dadd_rn(acc, __dmul_rn((double)vhi[s].w, chain));
		xprev = x;
	}
	double cm = __ddiv_rn(acc, mass[m]);
	if (cm > L) cm = __dsub_rn(cm, L);
	else if (cm < 0.0) cm = __dadd_rn(cm, L);
	return cm;
}

__global__ void k_mol_cmz(int nmol, const int *first, const int *nuau, const double *mass, const int4 *pos,
			  const uint4 *xlo, const int *inv, const float4 *vhi, double L, double *cmz)
{
	const int m = blockIdx.x * blockDim.x + threadIdx.x;
	if (m < nmol) cmz[m] = mol_cm_k(m, 2, first, nuau, mass, pos, xlo, inv, vhi, L);
}

__global__ void k_berendsen_mol(long n, int nmol, int4 *pos, uint4 *xlo, int4 *xn, int4 *cross, const int *mol,
				const double *cmz, double L0, double L1, double scale)
{
	const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
	if (i >= n) return;
	const int4 p = pos[i];
	const uint4 lo = xlo[i];
	const int m = mol[i];
	double x = from_fixed_dev((unsigned)p.z, lo.z, L0);
	int cr = 0;
	if (m >= 0 && m < nmol) {
		const double dr0 = __dsub_rn(x, cmz[m]);
		x = __dadd_rn(__dmul_rn(cmz[m], scale), dr0);
		if (x > L1) x = __dsub_rn(x, L1);
		else if (x < 0.0) x = __dadd_rn(x, L1);
	} else if (x >= L1) {
		x = __dsub_rn(x, L1);
		cr = 1;
	}
	unsigned h, l, hn, ln;
	to_fixed_dev(x, L1, h, l);
	pos[i] = make_int4(p.x, p.y, (int)h, p.w);
	xlo[i] = make_uint4(lo.x, lo.y, l, 0u);
	const int4 q = xn[i];
	to_fixed_dev(from_fixed_dev((unsigned)q.z, 0u, L0), L1, hn, ln);
	xn[i] = make_int4(q.x, q.y, (int)hn, q.w);
	if (cr) cross[i].z += 1;
}

extern void sepdev_runner_free(sepdev *d);

extern "C" int sepdev_berendsen_mol(sepdev *d, sepdev_moltab *t, double L1z, double scale)
{
	if (!(L1z > 0.0) || !(scale > 0.0) || !d->mol) return SEPDEV_EINVAL;
	double *cmz = t->props;      // scratch: nmol values
	const int4 *pos = d->pos[d->cur];
	k_mol_cmz<<<grid_for(t->nmol, 128), 128, 0, d->st>>>(t->nmol, t->first, t->nuau, t->mass, pos, d->xlo,
							    d->inv, d->vhi, d->L[2], cmz);
	k_berendsen_mol<<<grid_for(d->n, 256), 256, 0, d->st>>>(d->n, t->nmol, d->pos[d->cur], d->xlo, d->xn,
								d->cross, d->mol, cmz, d->L[2], L1z, scale);
	d->launches++;
	CKL(d);
	d->L[2] = L1z;
	d->fscale[2] = (float)(L1z / 4294967296.0);
	// captured loop graphs hold the old box's scale factors
	sepdev_runner_free(d);
	return SEPDEV_OK;
}

// ---- molecular mean square displacement (source/sepsampler.c:1958-2036) --------
//
// Per molecule of the sampled type: the centre of mass now, crossings
// counted from its jumps of more than half the box since the last sample
// (as the reference does), the displacement dr from the block's first
// sample; per block the sums of |dr|^2 and cos(k_j dr_x), FP64, fixed order.

struct sepdev_mmsd {
	double *prev, *pos0;   // [nmol][3]
	int *cross;            // [nmol][3]
	unsigned char *sel;    // [nmol] 1: the molecule has the sampled type
	double *kvec, *part, *sum;
	int nk, nblk;
};

__global__ void __launch_bounds__(MSB) k_mmsd(int nmol, const int *first, const int *nuau, const double *mass,
					       const int4 *pos, const uint4 *xlo, const int *inv, const float4 *vhi,
					       double L0, double L1, double L2, int reset, sepdev_mmsd m, double *part)
{
	extern __shared__ double red[];       // [MSB / 32][1 + nk]
	const int i = blockIdx.x * MSB + threadIdx.x;
	const int nf = 1 + m.nk;
	const double L[3] = {L0, L1, L2};
	double sd = 0.0, dr0 = 0.0;
	bool on = false;
	if (i < nmol) {
		double cm[3];
		for (int k = 0; k < 3; k++) cm[k] = mol_cm_k(i, k, first, nuau, mass, pos, xlo, inv, vhi, L[k]);
		if (reset)
			for (int k = 0; k < 3; k++) {
				m.prev[3 * i + k] = m.pos0[3 * i + k] = cm[k];
				m.cross[3 * i + k] = 0;
			}
		if (m.sel[i]) {
			on = true;
			double dr[3];
			for (int k = 0; k < 3; k++) {
				const double d = __dsub_rn(m.prev[3 * i + k], cm[k]);
				if (d > 0.5 * L[k]) m.cross[3 * i + k]++;
				else if (d < -0.5 * L[k]) m.cross[3 * i + k]--;
				dr[k] = __dsub_rn(__dadd_rn(cm[k], __dmul_rn((double)m.cross[3 * i + k], L[k])), m.pos0[3 * i + k]);
				m.prev[3 * i + k] = cm[k];
			}
			sd = __dadd_rn(__dadd_rn(__dmul_rn(dr[0], dr[0]), __dmul_rn(dr[1], dr[1])), __dmul_rn(dr[2], dr[2]));
			dr0 = dr[0];
		}
	}
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	for (int q = 0; q < nf; q++) {
		double x = on ? (q == 0 ? sd : cos(m.kvec[q - 1] * dr0)) : 0.0;
		for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
		if (lane == 0) red[wid * nf + q] = x;
	}
	__syncthreads();
	for (int q = threadIdx.x; q < nf; q += MSB) {
		double x = 0.0;
		for (int w = 0; w < MSB / 32; w++) x += red[w * nf + q];
		part[(long)blockIdx.x * nf + q] = x;
	}
}

__global__ void k_mmsd_rows(int nf, int nblk, const double *part, double *out)
{
	const int q = blockIdx.x * blockDim.x + threadIdx.x;
	if (q >= nf) return;
	double s = 0.0;
	for (int b = 0; b < nblk; b++) s += part[(long)b * nf + q];
	out[q] = s;
}

extern "C" void sepdev_mmsd_destroy(sepdev_mmsd *m)
{
	if (!m) return;
	void *b[] = {m->prev, m->pos0, m->cross, m->sel, m->kvec, m->part, m->sum};
	for (size_t k = 0; k < sizeof b / sizeof b[0]; k++)
		if (b[k]) cudaFree(b[k]);
	free(m);
}

extern "C" int sepdev_mmsd_create(sepdev *d, sepdev_moltab *t, int nk, const double *k, sepdev_mmsd **out)
{
	(void)d;
	*out = NULL;
	if (nk < 0 || (1 + nk) * (MSB / 32) * 8 > 40 * 1024) return SEPDEV_EINVAL;
	sepdev_mmsd *m = (sepdev_mmsd *)calloc(1, sizeof *m);
	if (!m) return SEPDEV_ENOMEM;
	m->nk = nk;
	m->nblk = (t->nmol + MSB - 1) / MSB;
	const int nm = t->nmol;
	cudaError_t e = cudaMalloc((void **)&m->prev, sizeof(double) * 3 * nm);
	if (e == cudaSuccess) e = cudaMalloc((void **)&m->pos0, sizeof(double) * 3 * nm);
	if (e == cudaSuccess) e = cudaMalloc((void **)&m->cross, sizeof(int) * 3 * nm);
	if (e == cudaSuccess) e = cudaMalloc((void **)&m->sel, nm);
	if (e == cudaSuccess) e = cudaMalloc((void **)&m->kvec, sizeof(double) * (nk > 0 ? nk : 1));
	if (e == cudaSuccess) e = cudaMalloc((void **)&m->part, sizeof(double) * (1 + nk) * m->nblk);
	if (e == cudaSuccess) e = cudaMalloc((void **)&m->sum, sizeof(double) * (1 + nk));
	if (e == cudaSuccess && nk > 0) e = cudaMemcpy(m->kvec, k, sizeof(double) * nk, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemset(m->cross, 0, sizeof(int) * 3 * nm);
	if (e != cudaSuccess) {
		sepdev_mmsd_destroy(m);
		sepdev_set_error("mmsd buffers", e);
		return SEPDEV_ENOMEM;
	}
	*out = m;
	return SEPDEV_OK;
}

// sel (host, nmol): 1 for the molecules of the sampled type; reset: the
// sample starts a block.  out (host, 1 + nk): sum |dr|^2, sum cos(k_j dr_x)
extern "C" int sepdev_mmsd_sample(sepdev *d, sepdev_moltab *t, sepdev_mmsd *m, const unsigned char *sel, int reset,
				  double *out)
{
	const int nf = 1 + m->nk;
	CK(cudaMemcpyAsync(m->sel, sel, t->nmol, cudaMemcpyHostToDevice, d->st));
	k_mmsd<<<m->nblk, MSB, sizeof(double) * nf * (MSB / 32), d->st>>>(
		t->nmol, t->first, t->nuau, t->mass, d->pos[d->cur], d->xlo, d->inv, d->vhi, d->L[0], d->L[1], d->L[2],
		reset, *m, m->part);
	k_mmsd_rows<<<grid_for(nf, 64), 64, 0, d->st>>>(nf, m->nblk, m->part, m->sum);
	d->launches++;
	CKL(d);
	CK(cudaMemcpyAsync(out, m->sum, sizeof(double) * nf, cudaMemcpyDeviceToHost, d->st));
	CK(cudaStreamSynchronize(d->st));
	return SEPDEV_OK;
}

// ---- molecular profiles (source/sepsampler.c:1571-1666) -------------------------
//
// Per molecule of the sampled type: the centre of mass (chain order, as
// the reference's sep_mol_spin takes it), velocity, spin about the centre
// of mass and inertia tensor; binned by the centre of mass along dir into
// 64-bit fixed-point sums (2^-32 units), so the order of the atomics does
// not matter: m v[dirvel], m, count, s (3), m v^2 over the other two
// components, the inertia tensor (9, row-major).

#define MPF 16

__global__ void __launch_bounds__(MSB) k_mprofs(int nmol, const int *first, const int *nuau, const int *start,
						 const int *atoms, const double *mass, const int *inv, const int4 *pos,
						 const uint4 *xlo, const float4 *vhi, const float4 *vlo, double L0,
						 double L1, double L2, const unsigned char *sel, int dir, int dirvel,
						 int lvec, unsigned long long *hist)
{
	const int m = blockIdx.x * MSB + threadIdx.x;
	if (m >= nmol || !sel[m]) return;
	const double L[3] = {L0, L1, L2};
	double cm[3];
	for (int k = 0; k < 3; k++) cm[k] = mol_cm_k(m, k, first, nuau, mass, pos, xlo, inv, vhi, L[k]);
	double v[3] = {0.0, 0.0, 0.0}, s[3] = {0.0, 0.0, 0.0}, I[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
	for (int q = start[m]; q < start[m + 1]; q++) {
		const int sl = inv[atoms[q]];
		const int4 p = pos[sl];
		const uint4 l = xlo[sl];
		const float4 vh = vhi[sl], vl = vlo[sl];
		const double ma = (double)vh.w;
		const double va[3] = {(double)vh.x + (double)vl.x, (double)vh.y + (double)vl.y,
				      (double)vh.z + (double)vl.z};
		double d[3];
		for (int k = 0; k < 3; k++) {
			double r = coord(p, l, k, L[k]) - cm[k];
			if (r > 0.5 * L[k]) r -= L[k];
			else if (r < -0.5 * L[k]) r += L[k];
			d[k] = r;
			v[k] += va[k] * ma;
		}
		const double pm[3] = {va[0] * ma, va[1] * ma, va[2] * ma};
		s[0] += d[1] * pm[2] - d[2] * pm[1];
		s[1] += d[2] * pm[0] - d[0] * pm[2];
		s[2] += d[0] * pm[1] - d[1] * pm[0];
		I[0] += ma * (d[1] * d[1] + d[2] * d[2]);
		I[4] += ma * (d[0] * d[0] + d[2] * d[2]);
		I[8] += ma * (d[0] * d[0] + d[1] * d[1]);
		I[1] -= ma * d[0] * d[1];
		I[2] -= ma * d[0] * d[2];
		I[5] -= ma * d[1] * d[2];
	}
	I[3] = I[1]; I[6] = I[2]; I[7] = I[5];
	const double M = mass[m];
	for (int k = 0; k < 3; k++) v[k] /= M;
	const double dl = L[dir] / lvec;
	int b = (int)(cm[dir] / dl);
	b = b < 0 ? 0 : (b >= lvec ? lvec - 1 : b);
	double t = 0.0;
	for (int k = 0; k < 3; k++)
		if (k != dirvel) t += M * v[k] * v[k];
	const double val[MPF] = {M * v[dirvel], M, 1.0, s[0], s[1], s[2], t,
				 I[0], I[1], I[2], I[3], I[4], I[5], I[6], I[7], I[8]};
	for (int q = 0; q < MPF; q++)
		atomicAdd(&hist[(long)b * MPF + q], (unsigned long long)llrint(ldexp(val[q], 32)));
}

// sel (host, nmol): the molecules of the sampled type; out (host, lvec x 16)
extern "C" int sepdev_mprofs(sepdev *d, sepdev_moltab *t, const unsigned char *sel, int dir, int dirvel, int lvec,
			     double *out)
{
	if (dir < 0 || dir > 2 || dirvel < 0 || dirvel > 2 || lvec < 1) return SEPDEV_EINVAL;
	unsigned long long *hist = NULL;
	unsigned char *dsel = NULL;
	cudaError_t e = cudaMalloc((void **)&hist, sizeof(long long) * MPF * lvec);
	if (e == cudaSuccess) e = cudaMalloc((void **)&dsel, t->nmol);
	if (e == cudaSuccess) e = cudaMemsetAsync(hist, 0, sizeof(long long) * MPF * lvec, d->st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(dsel, sel, t->nmol, cudaMemcpyHostToDevice, d->st);
	if (e != cudaSuccess) { cudaFree(hist); cudaFree(dsel); sepdev_set_error("mprofs", e); return SEPDEV_ECUDA; }
	k_mprofs<<<t->nblk, MSB, 0, d->st>>>(t->nmol, t->first, t->nuau, t->start, t->atoms, t->mass, d->inv,
					     d->pos[d->cur], d->xlo, d->vhi, d->vlo, d->L[0], d->L[1], d->L[2], dsel,
					     dir, dirvel, lvec, hist);
	CKL(d);
	long long *h = (long long *)malloc(sizeof(long long) * MPF * lvec);
	if (!h) { cudaFree(hist); cudaFree(dsel); return SEPDEV_ENOMEM; }
	e = cudaMemcpyAsync(h, hist, sizeof(long long) * MPF * lvec, cudaMemcpyDeviceToHost, d->st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
	cudaFree(hist); cudaFree(dsel);
	if (e != cudaSuccess) { free(h); sepdev_set_error("mprofs", e); return SEPDEV_ECUDA; }
	for (int k = 0; k < MPF * lvec; k++) out[k] = ldexp((double)h[k], -32);
	free(h);
	return SEPDEV_OK;
}

// ---- mavacf (source/sepsampler.c:1853-1906) ----------------------------------------
//
// The reference's sampled quantity: for each molecule of type A, the y
// component of the end-to-end vector from its atom 0 to its atom b (b the
// first molecule's atom count - 1; minimum image, source/sepmol.c:1106-1124)
// times the first particle's |charge| times the molecule mass; molecules of
// other types give 0.  A molecule with fewer atoms takes its last one.

__global__ void k_mol_ete_y(int nmol, const int *start, const int *atoms, const int *inv, const int4 *pos,
			    const uint4 *xlo, const double *mass, const unsigned char *sel, int b, double Ly,
			    double q, double *row)
{
	const int m = blockIdx.x * blockDim.x + threadIdx.x;
	if (m >= nmol) return;
	if (!sel[m]) { row[m] = 0.0; return; }
	const int last = start[m + 1] - 1;
	const int sa = inv[atoms[start[m]]], sb = inv[atoms[min(start[m] + b, last)]];
	double r = __dsub_rn(from_fixed_dev((unsigned)pos[sa].y, xlo[sa].y, Ly),
			     from_fixed_dev((unsigned)pos[sb].y, xlo[sb].y, Ly));
	if (r > 0.5 * Ly) r = __dsub_rn(r, Ly);
	else if (r < -0.5 * Ly) r = __dadd_rn(r, Ly);
	row[m] = r * q * mass[m];
}

// sel (host, nmol): the molecules of type A; q: |charge| of particle 0
extern "C" int sepdev_mavacf_store(sepdev *d, sepdev_moltab *t, sepdev_vacf *v, int index, const unsigned char *sel,
				   int b, double q)
{
	double *row = sepdev_vacf_row(v, index);
	if (!row || sepdev_vacf_count(v) != t->nmol) return SEPDEV_EINVAL;
	unsigned char *dsel = NULL;
	CK(cudaMalloc((void **)&dsel, t->nmol));
	cudaError_t e = cudaMemcpyAsync(dsel, sel, t->nmol, cudaMemcpyHostToDevice, d->st);
	if (e == cudaSuccess) {
		k_mol_ete_y<<<grid_for(t->nmol, 128), 128, 0, d->st>>>(t->nmol, t->start, t->atoms, d->inv, d->pos[d->cur],
								      d->xlo, t->mass, dsel, b, d->L[1], q, row);
		e = cudaGetLastError();
		d->launches++;
	}
	if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
	cudaFree(dsel);
	if (e != cudaSuccess) { sepdev_set_error("mavacf sample", e); return SEPDEV_ECUDA; }
	return SEPDEV_OK;
}
