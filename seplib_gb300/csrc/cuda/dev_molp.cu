// dev_molp.cu - the molecular pressure tensor without the molecular force
// matrix.
//
// The reference (source/sepmol.c:913-959) accumulates F[i][j], the force
// molecule j exerts on molecule i, over every pair force of a step (an
// nmol x nmol x 3 array), and at sep_mol_pressure_tensor forms
//     pot_P_mol = sum_{i<j} F[i][j] (x) R'_ij,
// R'_ij the minimum image of the centres of mass at that later call (after
// the integrator step, and after any box change).  For interacting
// molecules R'_ij = R_ij + dR_i - dR_j, R_ij taken at the pair pass and dR
// the change of a centre of mass since then, so
//     pot_P_mol = sum_{i<j} F[i][j] (x) R_ij + sum_i F_i (x) dR_i,
// F_i the total intermolecular force on molecule i.  The first sum is
// accumulated by the pair kernels atom pair by atom pair (k_pair<..., MOLV>);
// the second needs F_i per molecule, kept here as a per-atom intermolecular
// force.  Memory is O(N + nmol) instead of O(nmol^2).
//
// Centres of mass follow source/sepmol.c:683-729: the chain of consecutive
// user indices from the molecule's first atom, each bond unwrapped by the
// minimum image, mass-weighted, divided by the molecule mass.
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "dev_common.cuh"
#include "dev_pair.cuh"

#define MB 128

// centre of mass of molecule m as fixed-point high words
__device__ __forceinline__ int4 mol_cm(int m, const int *first, const int *nuau, const double *mass,
				       const int4 *pos, const int *inv, const float4 *vhi)
{
	const int a0 = first[m];
	const int4 p0 = pos[inv[a0]];
	long long off[3] = {0, 0, 0};
	double c[3] = {0.0, 0.0, 0.0};
	int4 prev = p0;
	for (int q = 0; q < nuau[m]; q++) {
		const int s = inv[a0 + q];
		const int4 p = pos[s];
		if (q > 0) {
			off[0] += (int)((unsigned)p.x - (unsigned)prev.x);
			off[1] += (int)((unsigned)p.y - (unsigned)prev.y);
			off[2] += (int)((unsigned)p.z - (unsigned)prev.z);
		}
		prev = p;
		const double ma = (double)vhi[s].w;
		c[0] += ma * (double)off[0]; c[1] += ma * (double)off[1]; c[2] += ma * (double)off[2];
	}
	const double im = 1.0 / mass[m];
	return make_int4((int)((unsigned)p0.x + (unsigned)llrint(c[0] * im)),
			 (int)((unsigned)p0.y + (unsigned)llrint(c[1] * im)),
			 (int)((unsigned)p0.z + (unsigned)llrint(c[2] * im)), 0);
}

__global__ void k_mol_cm(int nmol, const int *first, const int *nuau, const double *mass, const int4 *pos,
			 const int *inv, const float4 *vhi, int4 *cm)
{
	const int m = blockIdx.x * blockDim.x + threadIdx.x;
	if (m < nmol) cm[m] = mol_cm(m, first, nuau, mass, pos, inv, vhi);
}

struct MolpArgs {
	int nmol;
	const int *first, *nuau, *start, *atoms, *inv;
	const double *mass;
	const int4 *pos;
	const float4 *vhi, *vlo, *finter;
	const int4 *cm0;
	double L0[3], L1[3];
	double *out;            // [nmol][6]: centre of mass (wrapped), velocity
	double *part;           // [blocks][18]: kin (9), corr (9)
};

// per molecule: its centre of mass and velocity now, M v v^T and F_i (x) dR_i;
// block sums in a fixed order
__global__ void __launch_bounds__(MB) k_molp(MolpArgs a)
{
	__shared__ double red[MB];
	const int m = blockIdx.x * MB + threadIdx.x;
	double t[18];
	for (int k = 0; k < 18; k++) t[k] = 0.0;
	if (m < a.nmol) {
		const int4 c1 = mol_cm(m, a.first, a.nuau, a.mass, a.pos, a.inv, a.vhi);
		const int4 c0 = a.cm0[m];
		const unsigned h1[3] = {(unsigned)c1.x, (unsigned)c1.y, (unsigned)c1.z};
		const unsigned h0[3] = {(unsigned)c0.x, (unsigned)c0.y, (unsigned)c0.z};
		double v[3] = {0.0, 0.0, 0.0}, F[3] = {0.0, 0.0, 0.0}, dR[3];
		for (int q = a.start[m]; q < a.start[m + 1]; q++) {
			const int u = a.atoms[q], s = a.inv[u];
			const float4 vh = a.vhi[s], vl = a.vlo[s];
			const double ma = (double)vh.w;
			v[0] += ((double)vh.x + (double)vl.x) * ma;
			v[1] += ((double)vh.y + (double)vl.y) * ma;
			v[2] += ((double)vh.z + (double)vl.z) * ma;
			const float4 f = a.finter[u];
			F[0] += f.x; F[1] += f.y; F[2] += f.z;
		}
		const double M = a.mass[m];
		for (int k = 0; k < 3; k++) {
			v[k] /= M;
			// dR = L1 (f1 - f0) + (L1 - L0) f0, fractions f of the box
			const double df = ldexp((double)(int)(h1[k] - h0[k]), -32), f0 = ldexp((double)h0[k], -32);
			dR[k] = a.L1[k] * df + (a.L1[k] - a.L0[k]) * f0;
			a.out[6 * m + k] = ldexp((double)h1[k], -32) * a.L1[k];
			a.out[6 * m + 3 + k] = v[k];
		}
		for (int k = 0; k < 3; k++)
			for (int kk = 0; kk < 3; kk++) {
				t[3 * k + kk] = M * v[k] * v[kk];
				t[9 + 3 * k + kk] = F[k] * dR[kk];
			}
	}
	for (int k = 0; k < 18; k++) {
		red[threadIdx.x] = t[k];
		__syncthreads();
		for (int s = MB / 2; s > 0; s >>= 1) {
			if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
			__syncthreads();
		}
		if (threadIdx.x == 0) a.part[(long)blockIdx.x * 18 + k] = red[0];
		__syncthreads();
	}
}

// ---- host side ---------------------------------------------------------------

static void molvir_free(sepdev *d)
{
	void *b[] = {d->mv_first, d->mv_nuau, d->mv_start, d->mv_atoms, d->mv_mass, d->mv_cm,
		     d->mv_finter, d->mv_out};
	for (size_t k = 0; k < sizeof b / sizeof b[0]; k++)
		if (b[k]) cudaFree(b[k]);
	d->mv_first = d->mv_nuau = d->mv_start = d->mv_atoms = NULL;
	d->mv_mass = NULL; d->mv_cm = NULL; d->mv_finter = NULL; d->mv_out = NULL;
	d->molvir_on = 0;
	d->nmolv = 0;
}

extern void sepdev_runner_free(sepdev *d);

extern "C" int sepdev_molvir_enable(sepdev *d, int nmol, const int *first, const int *nuau,
				    const int *start, const int *atoms, const double *mass)
{
	if (nmol < 1) return SEPDEV_EINVAL;
	for (int m = 0; m < nmol; m++)
		if (nuau[m] < 1 || first[m] < 0 || first[m] + nuau[m] > d->n) return SEPDEV_EINVAL;
	for (int q = 0; q < start[nmol]; q++)
		if (atoms[q] < 0 || atoms[q] >= d->n) return SEPDEV_EINVAL;
	molvir_free(d);
	const int nblk = (nmol + MB - 1) / MB;
	cudaError_t e = cudaMalloc((void **)&d->mv_first, sizeof(int) * nmol);
	if (e == cudaSuccess) e = cudaMalloc((void **)&d->mv_nuau, sizeof(int) * nmol);
	if (e == cudaSuccess) e = cudaMalloc((void **)&d->mv_start, sizeof(int) * (nmol + 1));
	if (e == cudaSuccess) e = cudaMalloc((void **)&d->mv_atoms, sizeof(int) * (start[nmol] > 0 ? start[nmol] : 1));
	if (e == cudaSuccess) e = cudaMalloc((void **)&d->mv_mass, sizeof(double) * nmol);
	if (e == cudaSuccess) e = cudaMalloc((void **)&d->mv_cm, sizeof(int4) * nmol);
	if (e == cudaSuccess) e = cudaMalloc((void **)&d->mv_finter, sizeof(float4) * d->n);
	if (e == cudaSuccess) e = cudaMalloc((void **)&d->mv_out, sizeof(double) * (6 * nmol + 18 * nblk));
	if (e == cudaSuccess) e = cudaMemcpy(d->mv_first, first, sizeof(int) * nmol, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(d->mv_nuau, nuau, sizeof(int) * nmol, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(d->mv_start, start, sizeof(int) * (nmol + 1), cudaMemcpyHostToDevice);
	if (e == cudaSuccess && start[nmol] > 0)
		e = cudaMemcpy(d->mv_atoms, atoms, sizeof(int) * start[nmol], cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(d->mv_mass, mass, sizeof(double) * nmol, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemset(d->mv_cm, 0, sizeof(int4) * nmol);
	if (e == cudaSuccess) e = cudaMemset(d->mv_finter, 0, sizeof(float4) * d->n);
	if (e != cudaSuccess) {
		molvir_free(d);
		sepdev_set_error("molecular tables", e);
		return SEPDEV_ENOMEM;
	}
	d->nmolv = nmol;
	d->molvir_on = 1;
	d->mv_slot = -1;
	for (int k = 0; k < 3; k++) d->mv_L[k] = d->L[k];
	// loop graphs captured earlier launch the pair kernels without it
	sepdev_runner_free(d);
	return SEPDEV_OK;
}

extern "C" void sepdev_molvir_disable(sepdev *d)
{
	if (d->molvir_on) sepdev_runner_free(d);
	molvir_free(d);
}

extern "C" int sepdev_molvir_slot(sepdev *d, int slot)
{
	if (slot < 0 || slot >= d->nslots) return SEPDEV_EINVAL;
	d->mv_slot = slot;
	return SEPDEV_OK;
}

extern "C" int sepdev_molvir_reset(sepdev *d)
{
	if (!d->molvir_on) return SEPDEV_OK;
	CK(cudaMemsetAsync(d->mv_finter, 0, sizeof(float4) * d->n, d->st));
	return SEPDEV_OK;
}

int sepdev_molvir_cm(sepdev *d, const int4 *pos)
{
	k_mol_cm<<<(d->nmolv + MB - 1) / MB, MB, 0, d->st>>>(d->nmolv, d->mv_first, d->mv_nuau, d->mv_mass,
								pos, d->inv, d->vhi, d->mv_cm);
	CKL(d);
	for (int k = 0; k < 3; k++) d->mv_L[k] = d->L[k];
	return SEPDEV_OK;
}

extern "C" int sepdev_mol_state(sepdev *d, double *kin, double *corr, double *cm, double *vcm, double *L0,
				double *L1)
{
	for (int k = 0; k < 3; k++) {
		if (L0) L0[k] = d->mv_L[k];
		if (L1) L1[k] = d->L[k];
	}
	if (!d->molvir_on) return SEPDEV_EINVAL;
	const int nmol = d->nmolv, nblk = (nmol + MB - 1) / MB;
	MolpArgs a;
	a.nmol = nmol;
	a.first = d->mv_first; a.nuau = d->mv_nuau; a.start = d->mv_start; a.atoms = d->mv_atoms;
	a.inv = d->inv; a.mass = d->mv_mass;
	a.pos = d->pos[d->cur]; a.vhi = d->vhi; a.vlo = d->vlo; a.finter = d->mv_finter;
	a.cm0 = d->mv_cm;
	for (int k = 0; k < 3; k++) { a.L0[k] = d->mv_L[k]; a.L1[k] = d->L[k]; }
	a.out = d->mv_out;
	a.part = d->mv_out + 6 * (long)nmol;
	k_molp<<<nblk, MB, 0, d->st>>>(a);
	CKL(d);
	double *h = (double *)malloc(sizeof(double) * (6 * nmol + 18 * nblk));
	if (!h) return SEPDEV_ENOMEM;
	cudaError_t e = cudaMemcpyAsync(h, d->mv_out, sizeof(double) * (6 * nmol + 18 * nblk),
					cudaMemcpyDeviceToHost, d->st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
	if (e != cudaSuccess) { free(h); sepdev_set_error("molecular state", e); return SEPDEV_ECUDA; }
	for (int k = 0; k < 9; k++) { kin[k] = 0.0; corr[k] = 0.0; }
	for (int b = 0; b < nblk; b++)
		for (int k = 0; k < 9; k++) {
			kin[k] += h[6 * nmol + 18 * b + k];
			corr[k] += h[6 * nmol + 18 * b + 9 + k];
		}
	for (int m = 0; m < nmol; m++)
		for (int k = 0; k < 3; k++) {
			if (cm) cm[3 * m + k] = h[6 * m + k];
			if (vcm) vcm[3 * m + k] = h[6 * m + 3 + k];
		}
	free(h);
	return SEPDEV_OK;
}
