// dev_stoch.cu - stochastic dynamics: the DPD pair force of Groot and Warren,
// their velocity-Verlet integrator, the Fokker-Planck (Brownian) integrator
// and the Langevin integrator of Gronbech-Jensen and Farago (GJF), with the
// random numbers they draw.
//
// Reference semantics restated here:
//   DPD pair force       source/sepprfrc.c:1007-1104 (list), :1134-1235 (O(N^2))
//   Groot-Warren step    source/sepintgr.c:296-345
//   Fokker-Planck step   source/sepintgr.c:235-293
//   GJF Langevin step    source/sepintgr.c:91-146
//
// Random numbers.  The reference draws from the C library's rand() in the
// order its serial loops run.  Here every draw is a pure function of what it
// is drawn for: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) of a
// counter that names the pair or particle (user indices), the call and the
// stream, keyed by the run's seed.  A pair's number depends on its two user
// indices only, so the two sides of the full neighbour list apply the same
// random force and Newton's third law holds exactly; results depend neither
// on the particle order nor on the launch shape.
//
// Number formats as in the rest of the library: FP32 pair terms, float-float
// velocities, 64-bit fixed-point positions (increments through ff_mul_fix),
// exact fixed-point sums over particles.
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "dev_common.cuh"
#include "dev_pair.cuh"

#define SB 256

__device__ __forceinline__ void philox10(uint32_t (&c)[4], uint32_t k0, uint32_t k1)
{
#pragma unroll
	for (int r = 0; r < 10; r++) {
		if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
		const uint32_t h0 = __umulhi(0xD2511F53u, c[0]), l0 = 0xD2511F53u * c[0];
		const uint32_t h1 = __umulhi(0xCD9E8D57u, c[2]), l1 = 0xCD9E8D57u * c[2];
		const uint32_t n0 = h1 ^ c[1] ^ k0, n2 = h0 ^ c[3] ^ k1;
		c[0] = n0; c[1] = l1; c[2] = n2; c[3] = l0;
	}
}

enum { STREAM_DPD = 1, STREAM_FP = 2, STREAM_GJF = 3 };

// three standard normals of particle gid (Box-Muller on the output pairs)
__device__ __forceinline__ void gauss3(uint32_t k0, uint32_t k1, int gid, uint32_t call, uint32_t stream,
				       float (&g)[3])
{
	uint32_t c[4] = {(uint32_t)gid, 0u, call, stream};
	philox10(c, k0, k1);
	const float s24 = 1.0f / 16777216.0f;
	float sn, cs;
	const float r0 = sqrtf(-2.0f * logf((float)((c[0] >> 8) + 1u) * s24));
	sincospif(2.0f * (float)(c[1] >> 8) * s24, &sn, &cs);
	g[0] = r0 * cs;
	g[1] = r0 * sn;
	const float r1 = sqrtf(-2.0f * logf((float)((c[2] >> 8) + 1u) * s24));
	g[2] = r1 * cospif(2.0f * (float)(c[3] >> 8) * s24);
}

// ---- DPD pair force ----------------------------------------------------------

struct DpdArgs {
	const int4 *pos;
	const int *gid;
	const float4 *pv;
	float4 *frc;
	const int *nl;
	const int *ncnt;
	int maxnb;
	float fs[3];
	int tA, tB;
	float cf2, aij, gamma, sig_isdt;     // sig_isdt = sigma / sqrt(dt)
	uint32_t k0, k1, call;
	int accumulate;
	long long *slot;
	int off2;                            // slot2 - slot, in fields
	// molecular sums (MOLV): molecule of each slot, centres of mass at the
	// pass, per-atom intermolecular force (user order), mslot - slot
	const int *mol;
	const int4 *mcm;
	float4 *finter;
	int moff;
};

// Full list: particle i sums the pair terms of all its neighbours.  The
// per-side energy is aij w^2 / 4 (each pair is seen from both ends).  VIR:
// the O(N^2) form also accumulates the conservative, random and dissipative
// virials f_k r_kk (halved for the same reason).  MOLV (with VIR): the
// conservative force of each pair of atoms in different molecules also
// adds f (x) R_ij and f (x) n_ij to the molecular slot and f to the atom's
// intermolecular force, as the pair kernels do for their forces (the
// reference's O(N^2) form adds the conservative force to its molecular
// force matrix, source/sepprfrc.c:1211-1222).
template <bool VIR, bool MOLV = false>
__global__ void __launch_bounds__(SB) k_dpd(long n, DpdArgs a)
{
	const long i = blockIdx.x * (long)SB + threadIdx.x;
	float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
	float wc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, wr[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
	float wd[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
	float wm[18];
#pragma unroll
	for (int k = 0; k < 18; k++) wm[k] = 0.f;
	float gix = 0.f, giy = 0.f, giz = 0.f;
	int mi = -1;
	if (i < n) {
		const int4 pi = a.pos[i];
		int4 ci = make_int4(0, 0, 0, 0);
		if (MOLV) {
			mi = a.mol[i];
			if (mi >= 0) ci = a.mcm[mi];
		}
		if (pi.w == a.tA || pi.w == a.tB) {
			const float4 vi = a.pv[i];
			const int gi = a.gid[i], cnt = a.ncnt[i];
			const int tO = pi.w == a.tA ? a.tB : a.tA;    // the partner type
			const int *lp = a.nl + nl_index(i, 0, a.maxnb);
			for (int k = 0; k < cnt; k++) {
				const int j = __ldg(lp + (k >> 2) * 128 + (k & 3));
				const int4 pj = __ldg(&a.pos[j]);
				if (pj.w != tO) continue;
				const float dx = sep_hi(pi.x, pj.x, a.fs[0]);
				const float dy = sep_hi(pi.y, pj.y, a.fs[1]);
				const float dz = sep_hi(pi.z, pj.z, a.fs[2]);
				const float r2 = dx * dx + dy * dy + dz * dz;
				if (!(r2 < a.cf2)) continue;
				const float dij = sqrtf(r2), w = 1.0f - dij, id = 1.0f / dij;
				const float rx = dx * id, ry = dy * id, rz = dz * id;
				const float4 vj = __ldg(&a.pv[j]);
				const float dotrv = rx * (vi.x - vj.x) + ry * (vi.y - vj.y) + rz * (vi.z - vj.z);
				const int gj = __ldg(&a.gid[j]);
				uint32_t c[4] = {(uint32_t)min(gi, gj), (uint32_t)max(gi, gj), a.call, STREAM_DPD};
				philox10(c, a.k0, a.k1);
				const float rn = ((float)(c[0] >> 8) * (1.0f / 16777216.0f) - 0.5f) * 3.46410162f;
				const float fc = a.aij * w, fd = -a.gamma * w * w * dotrv, fr = a.sig_isdt * w * rn;
				const float s = fc + fd + fr;
				fx += s * rx; fy += s * ry; fz += s * rz;
				e += a.aij * w * w;
				if (VIR) {
					const float d[3] = {dx, dy, dz}, rh[3] = {rx, ry, rz};
					int q = 0;
#pragma unroll
					for (int p = 0; p < 3; p++)
#pragma unroll
						for (int r = p; r < 3; r++, q++) {
							const float rr = rh[p] * d[r];
							wc[q] += fc * rr; wr[q] += fr * rr; wd[q] += fd * rr;
						}
				}
				if (MOLV && mi >= 0) {
					const int mj = __ldg(&a.mol[j]);
					if (mj >= 0 && mj != mi) {
						const int4 cj = __ldg(&a.mcm[mj]);
						const unsigned hi[3] = {(unsigned)ci.x, (unsigned)ci.y, (unsigned)ci.z};
						const unsigned hj[3] = {(unsigned)cj.x, (unsigned)cj.y, (unsigned)cj.z};
						const float g3[3] = {fc * rx, fc * ry, fc * rz};
						float R[3], nim[3];
#pragma unroll
						for (int q = 0; q < 3; q++) {
							const int dI = (int)(hi[q] - hj[q]);
							R[q] = (float)dI * a.fs[q];
							nim[q] = (float)((((long long)hi[q] - (long long)hj[q]) - dI) >> 32);
						}
#pragma unroll
						for (int p = 0; p < 3; p++)
#pragma unroll
							for (int q = 0; q < 3; q++) {
								wm[3 * p + q] += g3[p] * R[q];
								wm[9 + 3 * p + q] += g3[p] * nim[q];
							}
						gix += g3[0]; giy += g3[1]; giz += g3[2];
					}
				}
			}
		}
		if (MOLV && mi >= 0) {
			const int u = a.gid[i];
			float4 fo = a.finter[u];
			fo.x += gix; fo.y += giy; fo.z += giz;
			a.finter[u] = fo;
		}
		float4 f = a.accumulate ? a.frc[i] : make_float4(0.f, 0.f, 0.f, 0.f);
		f.x += fx; f.y += fy; f.z += fz;
		a.frc[i] = f;
	}
	if (VIR) {
		constexpr int NM = MOLV ? 18 : 0;
		float v[19 + NM];
		int fld[19 + NM];
		v[0] = 0.25f * e; fld[0] = SLOT_EPOT0;
		for (int q = 0; q < 6; q++) {
			v[1 + q] = 0.5f * wc[q]; fld[1 + q] = SLOT_POTP + q;
			v[7 + q] = 0.5f * wr[q]; fld[7 + q] = SLOT_POTPB + q;
			v[13 + q] = 0.5f * wd[q]; fld[13 + q] = a.off2 + SLOT_POTP + q;
		}
#pragma unroll
		for (int k = 0; k < NM; k++) { v[19 + k] = 0.5f * wm[k]; fld[19 + k] = a.moff + k; }
		block_to_slot<19 + NM>(v, fld, a.slot, 0.f, -1);
	} else {
		float v[1] = {0.25f * e};
		const int fld[1] = {SLOT_EPOT0};
		block_to_slot<1>(v, fld, a.slot, 0.f, -1);
	}
}

// ---- integrators -------------------------------------------------------------

struct StochArgs {
	int4 *pos;              // updated in place
	uint4 *xlo;
	float4 *vhi, *vlo;
	const float4 *frc;
	float4 *ext[SEPDEV_NEXT];
	const int *gid;
	const int4 *xn;
	int4 *cross;
	float fs[3], shi[3], slo[3];
	float dt;
	// Groot-Warren
	float lambda;
	int stepnow;
	// Fokker-Planck / GJF
	float temp, alpha, fac;
	uint32_t k0, k1, call;
	long long *slot;
};

// add 64-bit fixed-point increments to particle i's position, count the
// crossings, return the squared displacement from the last build's position
__device__ __forceinline__ float advance(long i, const StochArgs &a, const long long (&inc)[3])
{
	const int4 pi = a.pos[i];
	const uint4 lo = a.xlo[i];
	const unsigned hi[3] = {(unsigned)pi.x, (unsigned)pi.y, (unsigned)pi.z};
	const unsigned lw[3] = {lo.x, lo.y, lo.z};
	unsigned nh[3], nl[3];
	int cr[3];
#pragma unroll
	for (int k = 0; k < 3; k++) {
		const unsigned long long X0 = ((unsigned long long)hi[k] << 32) | lw[k];
		const unsigned long long X1 = X0 + (unsigned long long)inc[k];
		cr[k] = (inc[k] > 0 && X1 < X0) ? 1 : ((inc[k] < 0 && X1 > X0) ? -1 : 0);
		nh[k] = (unsigned)(X1 >> 32);
		nl[k] = (unsigned)X1;
	}
	if (cr[0] | cr[1] | cr[2]) {
		int4 c = a.cross[i];
		c.x += cr[0]; c.y += cr[1]; c.z += cr[2];
		a.cross[i] = c;
	}
	const int4 po = make_int4((int)nh[0], (int)nh[1], (int)nh[2], pi.w);
	a.pos[i] = po;
	a.xlo[i] = make_uint4(nl[0], nl[1], nl[2], 0u);
	const int4 xn = a.xn[i];
	const float dx = sep_hi(po.x, xn.x, a.fs[0]);
	const float dy = sep_hi(po.y, xn.y, a.fs[1]);
	const float dz = sep_hi(po.z, xn.z, a.fs[2]);
	return dx * dx + dy * dy + dz * dz;
}

__device__ __forceinline__ void kin_terms(float m, float vx, float vy, float vz, float &ek, float (&kp)[6])
{
	ek = m * (vx * vx + vy * vy + vz * vz);
	kp[0] = m * vx * vx; kp[1] = m * vx * vy; kp[2] = m * vx * vz;
	kp[3] = m * vy * vy; kp[4] = m * vy * vz; kp[5] = m * vz * vz;
}

__device__ __forceinline__ void kin_to_slot(const StochArgs &a, float ek, float (&kp)[6], float d2)
{
	float v[8] = {ek, kp[0], kp[1], kp[2], kp[3], kp[4], kp[5], ek};
	const int fld[8] = {SLOT_EKIN, SLOT_KINP, SLOT_KINP + 1, SLOT_KINP + 2, SLOT_KINP + 3,
			    SLOT_KINP + 4, SLOT_KINP + 5, SLOT_SUMV2};
	block_to_slot<8>(v, fld, a.slot, d2, SLOT_MAXD2);
}

// a = f/m; v += dt (a + pa)/2 (not on step 0); x += dt (v + dt a/2);
// pv = v + lambda dt a; pa = a
__global__ void __launch_bounds__(SB) k_verlet_dpd(long n, StochArgs a)
{
	const long i = blockIdx.x * (long)SB + threadIdx.x;
	float ek = 0.f, kp[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, d2 = 0.f;
	if (i < n) {
		const float4 f = a.frc[i];
		float4 vh = a.vhi[i], vl = a.vlo[i];
		const float m = vh.w, im = vl.w, dt = a.dt;
		const float ac[3] = {f.x * im, f.y * im, f.z * im};
		const float4 pa = a.ext[SEPDEV_EXT_PA][i];
		float *h[3] = {&vh.x, &vh.y, &vh.z}, *l[3] = {&vl.x, &vl.y, &vl.z};
		const float pac[3] = {pa.x, pa.y, pa.z};
		long long inc[3];
		float pv[3];
#pragma unroll
		for (int k = 0; k < 3; k++) {
			if (a.stepnow > 0) ff_add(*h[k], *l[k], 0.5f * dt * (ac[k] + pac[k]));
			float uh = *h[k], ul = *l[k];
			ff_add(uh, ul, 0.5f * dt * ac[k]);
			inc[k] = ff_mul_fix(uh, ul, a.shi[k], a.slo[k]);
			pv[k] = *h[k] + (*l[k] + a.lambda * dt * ac[k]);
		}
		a.vhi[i] = vh;
		a.vlo[i] = vl;
		const float4 pvo = a.ext[SEPDEV_EXT_PV][i];
		a.ext[SEPDEV_EXT_PV][i] = make_float4(pv[0], pv[1], pv[2], pvo.w);
		a.ext[SEPDEV_EXT_PA][i] = make_float4(ac[0], ac[1], ac[2], 0.f);
		d2 = advance(i, a, inc);
		kin_terms(m, vh.x, vh.y, vh.z, ek, kp);
	}
	kin_to_slot(a, ek, kp, d2);
}

// fric = T / ldiff; x += dt v; v += dt/m (f - fric v + g sqrt(2 T fric / dt))
__global__ void __launch_bounds__(SB) k_fp(long n, StochArgs a)
{
	const long i = blockIdx.x * (long)SB + threadIdx.x;
	float ek = 0.f, kp[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, d2 = 0.f;
	if (i < n) {
		const float4 f = a.frc[i];
		float4 vh = a.vhi[i], vl = a.vlo[i];
		const float m = vh.w, im = vl.w, dt = a.dt;
		const float fric = a.temp / a.ext[SEPDEV_EXT_PV][i].w;
		// sqrt(1/12) sqrt(24 T fric / dt), as the reference writes it
		const float amp = sqrtf(1.0f / 12.0f) * sqrtf(24.0f * a.temp * fric / dt);
		float g[3];
		gauss3(a.k0, a.k1, a.gid[i], a.call, STREAM_FP, g);
		const float fc[3] = {f.x, f.y, f.z};
		float *h[3] = {&vh.x, &vh.y, &vh.z}, *l[3] = {&vl.x, &vl.y, &vl.z};
		long long inc[3];
#pragma unroll
		for (int k = 0; k < 3; k++) {
			inc[k] = ff_mul_fix(*h[k], *l[k], a.shi[k], a.slo[k]);     // the old velocity
			ff_add(*h[k], *l[k], im * dt * (fc[k] - fric * *h[k] + g[k] * amp));
		}
		a.vhi[i] = vh;
		a.vlo[i] = vl;
		d2 = advance(i, a, inc);
		kin_terms(m, vh.x, vh.y, vh.z, ek, kp);
	}
	kin_to_slot(a, ek, kp, d2);
}

// c = alpha dt / (2m), a' = (1-c)/(1+c), b = 1/(1+c):
// v = a' v + dt/(2m) (a' prevf + f) + b randn / m; prevf = f;
// randn = fac g (fac = sqrt(T (1 - exp(-2 alpha dt))));
// x += b dt (v + dt f/(2m) + randn/(2m))
__global__ void __launch_bounds__(SB) k_gjf(long n, StochArgs a)
{
	const long i = blockIdx.x * (long)SB + threadIdx.x;
	float ek = 0.f, kp[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, d2 = 0.f;
	if (i < n) {
		const float4 f = a.frc[i];
		float4 vh = a.vhi[i], vl = a.vlo[i];
		const float m = vh.w, im = vl.w, dt = a.dt;
		const float c = a.alpha * dt * 0.5f * im, ic = 1.0f / (1.0f + c);
		const float ap = (1.0f - c) * ic, am1 = -2.0f * c * ic, bm1 = -c * ic, b = ic;
		const float4 pf = a.ext[SEPDEV_EXT_PREVF][i], ro = a.ext[SEPDEV_EXT_RANDN][i];
		float g[3];
		gauss3(a.k0, a.k1, a.gid[i], a.call, STREAM_GJF, g);
		const float fc[3] = {f.x, f.y, f.z}, pfc[3] = {pf.x, pf.y, pf.z}, roc[3] = {ro.x, ro.y, ro.z};
		float *h[3] = {&vh.x, &vh.y, &vh.z}, *l[3] = {&vl.x, &vl.y, &vl.z};
		long long inc[3];
		float rn[3];
#pragma unroll
		for (int k = 0; k < 3; k++) {
			// a' v = v + (a' - 1) v keeps the float-float velocity exact in v
			ff_add(*h[k], *l[k], am1 * *h[k] + 0.5f * dt * im * (ap * pfc[k] + fc[k]) + b * im * roc[k]);
			rn[k] = a.fac * g[k];
			float uh = *h[k], ul = *l[k];
			ff_add(uh, ul, 0.5f * im * (dt * fc[k] + rn[k]));
			ff_add(uh, ul, bm1 * uh);                   // times b = 1 - c/(1+c)
			inc[k] = ff_mul_fix(uh, ul, a.shi[k], a.slo[k]);
		}
		a.vhi[i] = vh;
		a.vlo[i] = vl;
		a.ext[SEPDEV_EXT_PREVF][i] = make_float4(f.x, f.y, f.z, 0.f);
		a.ext[SEPDEV_EXT_RANDN][i] = make_float4(rn[0], rn[1], rn[2], 0.f);
		d2 = advance(i, a, inc);
		kin_terms(m, vh.x, vh.y, vh.z, ek, kp);
	}
	kin_to_slot(a, ek, kp, d2);
}

// ---- user-order transfers of the stochastic fields ---------------------------

__global__ void k_ext_scatter(long n, const int *inv, const float4 *src, float4 *dst)
{
	const long u = blockIdx.x * (long)blockDim.x + threadIdx.x;
	if (u < n) dst[inv[u]] = src[u];
}

__global__ void k_ext_gather(long n, const int *inv, const float4 *src, float4 *dst)
{
	const long u = blockIdx.x * (long)blockDim.x + threadIdx.x;
	if (u < n) dst[u] = src[inv[u]];
}

// ---- host side ---------------------------------------------------------------

extern void sepdev_runner_free(sepdev *d);

extern "C" int sepdev_ext_enabled(const sepdev *d)
{
	return d->ext[0] != NULL;
}

extern "C" int sepdev_ext_enable(sepdev *d)
{
	if (d->ext[0]) return SEPDEV_OK;
	const size_t bytes = sizeof(float4) * d->n;
	for (int k = 0; k < SEPDEV_NEXT; k++) {
		cudaError_t e = cudaMalloc((void **)&d->ext[k], bytes);
		if (e == cudaSuccess) e = cudaMalloc((void **)&d->ext_b[k], bytes);
		if (e == cudaSuccess) e = cudaMemsetAsync(d->ext[k], 0, bytes, d->st);
		if (e != cudaSuccess) {
			for (int q = 0; q <= k; q++) {
				cudaFree(d->ext[q]); cudaFree(d->ext_b[q]);
				d->ext[q] = d->ext_b[q] = NULL;
			}
			sepdev_set_error("stochastic fields", e);
			return SEPDEV_ENOMEM;
		}
	}
	// captured loop graphs permute the particle arrays they knew of
	sepdev_runner_free(d);
	return SEPDEV_OK;
}

extern "C" int sepdev_ext_upload(sepdev *d, const double *pv, const double *pa, const double *prevf,
				 const double *randn, const double *ldiff)
{
	if (!d->ext[0] || !pv || !pa || !prevf || !randn || !ldiff) return SEPDEV_EINVAL;
	const long n = d->n;
	float4 *h = (float4 *)malloc(sizeof(float4) * n);
	if (!h) return SEPDEV_ENOMEM;
	const double *src[SEPDEV_NEXT] = {pv, pa, prevf, randn};
	int rc = SEPDEV_OK;
	for (int k = 0; k < SEPDEV_NEXT && rc == SEPDEV_OK; k++) {
		for (long u = 0; u < n; u++)
			h[u] = make_float4((float)src[k][3 * u], (float)src[k][3 * u + 1], (float)src[k][3 * u + 2],
					   k == SEPDEV_EXT_PV ? (float)ldiff[u] : 0.f);
		cudaError_t e = cudaMemcpyAsync(d->ext_b[k], h, sizeof(float4) * n, cudaMemcpyHostToDevice, d->st);
		if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
		if (e != cudaSuccess) { sepdev_set_error("stochastic upload", e); rc = SEPDEV_ECUDA; break; }
		k_ext_scatter<<<grid_for(n, SB), SB, 0, d->st>>>(n, d->inv, d->ext_b[k], d->ext[k]);
		d->launches++;
		if ((e = cudaGetLastError()) != cudaSuccess) { sepdev_set_error("kernel launch", e); rc = SEPDEV_ECUDA; }
	}
	free(h);
	return rc;
}

extern "C" int sepdev_ext_download(sepdev *d, double *pv, double *pa, double *prevf, double *randn)
{
	if (!d->ext[0]) return SEPDEV_EINVAL;
	const long n = d->n;
	float4 *h = (float4 *)malloc(sizeof(float4) * n);
	if (!h) return SEPDEV_ENOMEM;
	double *dst[SEPDEV_NEXT] = {pv, pa, prevf, randn};
	int rc = SEPDEV_OK;
	for (int k = 0; k < SEPDEV_NEXT && rc == SEPDEV_OK; k++) {
		if (!dst[k]) continue;
		k_ext_gather<<<grid_for(n, SB), SB, 0, d->st>>>(n, d->inv, d->ext[k], d->ext_b[k]);
		d->launches++;
		cudaError_t e = cudaGetLastError();
		if (e == cudaSuccess)
			e = cudaMemcpyAsync(h, d->ext_b[k], sizeof(float4) * n, cudaMemcpyDeviceToHost, d->st);
		if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
		if (e != cudaSuccess) { sepdev_set_error("stochastic download", e); rc = SEPDEV_ECUDA; break; }
		for (long u = 0; u < n; u++) {
			dst[k][3 * u] = h[u].x; dst[k][3 * u + 1] = h[u].y; dst[k][3 * u + 2] = h[u].z;
		}
	}
	free(h);
	return rc;
}

extern "C" int sepdev_dpd_forces(sepdev *d, const sepdev_dpd *p, int accumulate, int slot, int slot2)
{
	if (!d->ext[0] || !d->list_valid) return SEPDEV_EINVAL;
	if (sepdev_list_confirm(d)) return SEPDEV_ECUDA;
	if (slot < 0 || slot >= d->nslots || (p->virial && (slot2 < 0 || slot2 >= d->nslots)))
		return SEPDEV_EINVAL;
	const bool molv = p->virial && p->mslot >= 0 && d->molvir_on;
	if (molv && p->mslot >= d->nslots) return SEPDEV_EINVAL;
	DpdArgs a;
	memset(&a, 0, sizeof a);
	a.pos = d->pos[d->cur];
	a.gid = d->gid;
	a.pv = d->ext[SEPDEV_EXT_PV];
	a.frc = d->frc;
	a.nl = d->nl; a.ncnt = d->ncnt; a.maxnb = d->maxnb;
	for (int k = 0; k < 3; k++) a.fs[k] = d->fscale[k];
	a.tA = p->tA; a.tB = p->tB;
	a.cf2 = (float)(p->cf * p->cf);
	a.aij = (float)p->aij;
	a.gamma = (float)p->gamma;
	a.sig_isdt = (float)(p->sigma / sqrt(p->dt));
	a.k0 = (uint32_t)p->seed; a.k1 = (uint32_t)(p->seed >> 32);
	a.call = p->call;
	a.accumulate = accumulate;
	a.slot = d->slots + (long)slot * SLOT_FIELDS;
	a.off2 = (slot2 - slot) * SLOT_FIELDS;
	if (molv) {
		// the centres of mass of this pass, as the pair passes take them
		sepdev_molvir_cm(d, a.pos);
		a.mol = d->mol;
		a.mcm = d->mv_cm;
		a.finter = d->mv_finter;
		a.moff = (p->mslot - slot) * SLOT_FIELDS;
		k_dpd<true, true><<<grid_for(d->n, SB), SB, 0, d->st>>>(d->n, a);
	} else if (p->virial) {
		k_dpd<true><<<grid_for(d->n, SB), SB, 0, d->st>>>(d->n, a);
	} else {
		k_dpd<false><<<grid_for(d->n, SB), SB, 0, d->st>>>(d->n, a);
	}
	CKL(d);
	return SEPDEV_OK;
}

static int stoch_args(sepdev *d, StochArgs &a, double dt, int slot)
{
	if (!d->ext[0] || slot < 0 || slot >= d->nslots) return SEPDEV_EINVAL;
	memset(&a, 0, sizeof a);
	a.pos = d->pos[d->cur];
	a.xlo = d->xlo; a.vhi = d->vhi; a.vlo = d->vlo; a.frc = d->frc;
	for (int k = 0; k < SEPDEV_NEXT; k++) a.ext[k] = d->ext[k];
	a.gid = d->gid; a.xn = d->xn; a.cross = d->cross;
	for (int k = 0; k < 3; k++) {
		a.fs[k] = d->fscale[k];
		const double S = dt * 18446744073709551616.0 / d->L[k];
		a.shi[k] = (float)S;
		a.slo[k] = (float)(S - (double)a.shi[k]);
	}
	a.dt = (float)dt;
	a.slot = d->slots + (long)slot * SLOT_FIELDS;
	return SEPDEV_OK;
}

extern "C" int sepdev_verlet_dpd(sepdev *d, double dt, double lambda, int stepnow, int slot)
{
	StochArgs a;
	int rc = stoch_args(d, a, dt, slot);
	if (rc) return rc;
	a.lambda = (float)lambda;
	a.stepnow = stepnow;
	k_verlet_dpd<<<grid_for(d->n, SB), SB, 0, d->st>>>(d->n, a);
	CKL(d);
	return SEPDEV_OK;
}

extern "C" int sepdev_fp(sepdev *d, double dt, double temp, unsigned long long seed, unsigned call, int slot)
{
	StochArgs a;
	int rc = stoch_args(d, a, dt, slot);
	if (rc) return rc;
	a.temp = (float)temp;
	a.k0 = (uint32_t)seed; a.k1 = (uint32_t)(seed >> 32); a.call = call;
	k_fp<<<grid_for(d->n, SB), SB, 0, d->st>>>(d->n, a);
	CKL(d);
	return SEPDEV_OK;
}

extern "C" int sepdev_gjf(sepdev *d, double dt, double temp, double alpha, unsigned long long seed,
			  unsigned call, int slot)
{
	StochArgs a;
	int rc = stoch_args(d, a, dt, slot);
	if (rc) return rc;
	const double cc = exp(-alpha * dt);
	a.temp = (float)temp;
	a.alpha = (float)alpha;
	a.fac = (float)sqrt(temp * (1.0 - cc * cc));
	a.k0 = (uint32_t)seed; a.k1 = (uint32_t)(seed >> 32); a.call = call;
	k_gjf<<<grid_for(d->n, SB), SB, 0, d->st>>>(d->n, a);
	CKL(d);
	return SEPDEV_OK;
}
