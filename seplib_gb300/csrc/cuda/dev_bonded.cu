// dev_bonded.cu - harmonic bonds, angles and Ryckaert-Bellemans torsions.
//
// Reference formulas: source/sepmol.c:372-415 (stretch), :418-466 (cos^2
// angle), :469-517 (harmonic angle), :520-587 (torsion, Rapaport's form).
//
// The reference loops over terms and scatters into both/all atoms.  Here
// every atom gathers: one thread per particle walks the terms it belongs to
// (an incidence CSR built once from the topology) and computes its own share
// of each term, so the force array sees no atomics.  The bonded calls of a
// step are deferred and evaluated together, one pending term per kind, in
// one launch.  Each term is evaluated
// by every member atom from bit-identical inputs, so the shares cancel
// exactly; energy, virial and the per-term observable are taken from the
// role-0 atom only.  Separations come from the full 64-bit fixed-point
// difference, so stiff bonds lose no precision to the box size.
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "dev_common.cuh"

#define TERM_BOND 0
#define TERM_ANGLE 1
#define TERM_DIHED 2
#define ENC(kind, role, idx) (((unsigned)(kind) << 30) | ((unsigned)(role) << 27) | (unsigned)(idx))

// One launch evaluates up to one pending term of each kind (bond, angle,
// torsion) with its own parameters and accumulator slot.
struct BondArgs {
	const int4 *pos;
	const uint4 *xlo;
	float4 *frc;
	const int *gid, *inv;
	const int *inc_start, *inc_term;
	const uint4 *bonds, *angles, *diheds;
	const int *dtype;
	float *term_out;
	long term_off[3];
	float fs[3];
	int has[3], type[3];
	float bl0, bk;        // bonds: l0, k
	float ap0, ak;        // angles: theta0 (or cos(pi - theta0)), k
	int cossq;
	float g[6];           // torsions
	int fld0[3];          // first accumulator field of each kind's slot
	int accumulate;       // add to the stored forces (else store)
	long long *slots;
};

// minimum-image separation x_a - x_b from the full fixed-point words
__device__ __forceinline__ float3 sep64(const BondArgs &a, int sa, int sb)
{
	const int4 ha = a.pos[sa], hb = a.pos[sb];
	const uint4 la = a.xlo[sa], lb = a.xlo[sb];
	const int hx[3] = {ha.x, ha.y, ha.z}, hy[3] = {hb.x, hb.y, hb.z};
	const unsigned lx[3] = {la.x, la.y, la.z}, ly[3] = {lb.x, lb.y, lb.z};
	float r[3];
#pragma unroll
	for (int k = 0; k < 3; k++) {
		const unsigned long long A = ((unsigned long long)(unsigned)hx[k] << 32) | lx[k];
		const unsigned long long B = ((unsigned long long)(unsigned)hy[k] << 32) | ly[k];
		const long long D = (long long)(A - B);
		const int dh = (int)(D >> 32);
		const unsigned dl = (unsigned)D;
		r[k] = (float)dh * a.fs[k] + (float)dl * (a.fs[k] * 2.3283064365386963e-10f);
	}
	return make_float3(r[0], r[1], r[2]);
}

__device__ __forceinline__ float dot3(float3 u, float3 w) { return u.x * w.x + u.y * w.y + u.z * w.z; }

// BOND_LPA lanes share a particle: each walks every BOND_LPA-th entry of its
// incidence list, and every incident term of a kind that is pending adds
// this atom's share; the lanes' forces are summed by shuffles in a fixed
// order.  One lane per particle measured fastest (4 lanes: 23.2 us against
// 14.0 us for 32000 butane beads: the extra warps' setup and block
// reductions cost more than the latency they hide).
#define BOND_LPA 1
__global__ void __launch_bounds__(256) k_bonded(long n, BondArgs a)
{
	const long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
	const long s = gt / BOND_LPA;
	const int sub = (int)(gt % BOND_LPA);
	float fx = 0.f, fy = 0.f, fz = 0.f, eb = 0.f, ea = 0.f, ed = 0.f;
	float w[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
	if (s < n) {
		const int u = a.gid[s];
		for (int t = a.inc_start[u] + sub, te = a.inc_start[u + 1]; t < te; t += BOND_LPA) {
			const unsigned code = (unsigned)a.inc_term[t];
			const int kind = (int)(code >> 30);
			if (!a.has[kind]) continue;
			const int role = (code >> 27) & 7;
			const int idx = code & ((1u << 27) - 1u);
			if (kind == TERM_BOND) {
				const uint4 b = a.bonds[idx];
				if ((int)b.z != a.type[0]) continue;
				const int sa = a.inv[b.x], sb = a.inv[b.y];
				const float3 r = sep64(a, sa, sb);
				const float r2 = dot3(r, r), dist = sqrtf(r2);
				const float ft = -a.bk * (dist - a.bl0) / dist;
				const float sg = role == 0 ? 1.f : -1.f;
				fx += sg * ft * r.x; fy += sg * ft * r.y; fz += sg * ft * r.z;
				if (role == 0) {
					eb += 0.5f * a.bk * (dist - a.bl0) * (dist - a.bl0);
					const float gx = ft * r.x, gy = ft * r.y, gz = ft * r.z;
					w[0] += gx * r.x; w[1] += gx * r.y; w[2] += gx * r.z;
					w[3] += gy * r.y; w[4] += gy * r.z; w[5] += gz * r.z;
					a.term_out[a.term_off[0] + idx] = dist;
				}
			} else if (kind == TERM_ANGLE) {
				const uint4 g = a.angles[idx];
				if ((int)g.w != a.type[1]) continue;
				const int sa = a.inv[g.x], sb = a.inv[g.y], sc = a.inv[g.z];
				const float3 d1 = sep64(a, sb, sa), d2 = sep64(a, sc, sb);
				const float c11 = dot3(d1, d1), c12 = dot3(d1, d2), c22 = dot3(d2, d2);
				const float cD = sqrtf(c11 * c22), cc = c12 / cD;
				float pref, th;
				if (a.cossq) {
					pref = -a.ak * (cc - a.ap0);
					th = 3.14159265358979f - acosf(fminf(fmaxf(cc, -1.f), 1.f));
					if (role == 0) ea += 0.5f * a.ak * (cc - a.ap0) * (cc - a.ap0);
				} else {
					th = 3.14159265358979f - acosf(fminf(fmaxf(cc, -1.f), 1.f));
					pref = -a.ak * (th - a.ap0);
					if (role == 0) ea += 0.5f * a.ak * (th - a.ap0) * (th - a.ap0);
				}
				const float q11 = c12 / c11, q22 = c12 / c22;
				const float3 f1 = make_float3(pref * (q11 * d1.x - d2.x) / cD, pref * (q11 * d1.y - d2.y) / cD,
							      pref * (q11 * d1.z - d2.z) / cD);
				const float3 f2 = make_float3(pref * (d1.x - q22 * d2.x) / cD, pref * (d1.y - q22 * d2.y) / cD,
							      pref * (d1.z - q22 * d2.z) / cD);
				if (role == 0) { fx += f1.x; fy += f1.y; fz += f1.z; a.term_out[a.term_off[1] + idx] = th; }
				else if (role == 1) { fx += -f1.x - f2.x; fy += -f1.y - f2.y; fz += -f1.z - f2.z; }
				else { fx += f2.x; fy += f2.y; fz += f2.z; }
			} else {
				const uint4 q = a.diheds[idx];
				if (a.dtype[idx] != a.type[2]) continue;
				const int sa = a.inv[q.x], sb = a.inv[q.y], sc = a.inv[q.z], sd = a.inv[q.w];
				const float3 r1 = sep64(a, sb, sa), r2 = sep64(a, sc, sb), r3 = sep64(a, sd, sc);
				const float c11 = dot3(r1, r1), c12 = dot3(r1, r2), c13 = dot3(r1, r3);
				const float c22 = dot3(r2, r2), c23 = dot3(r2, r3), c33 = dot3(r3, r3);
				const float cA = c13 * c22 - c12 * c23;
				const float cB1 = c11 * c22 - c12 * c12, cB2 = c22 * c33 - c23 * c23;
				const float cD = sqrtf(cB1 * cB2), cc = cA / cD;
				const float *gg = a.g;
				const float pref = -(gg[1] + (2.f * gg[2] + (3.f * gg[3] + (4.f * gg[4] + 5.f * gg[5] * cc) * cc) * cc) * cc);
				const float t1 = cA, t2 = c11 * c23 - c12 * c13, t3 = -cB1;
				const float t4 = cB2, t5 = c13 * c23 - c12 * c33, t6 = -cA;
				const float cR1 = c12 / c22, cR2 = c23 / c22;
				const float k1 = pref * c22 / (cD * cB1), k2 = pref * c22 / (cD * cB2);
				const float3 f1 = make_float3(k1 * (t1 * r1.x + t2 * r2.x + t3 * r3.x),
							      k1 * (t1 * r1.y + t2 * r2.y + t3 * r3.y),
							      k1 * (t1 * r1.z + t2 * r2.z + t3 * r3.z));
				const float3 f2 = make_float3(k2 * (t4 * r1.x + t5 * r2.x + t6 * r3.x),
							      k2 * (t4 * r1.y + t5 * r2.y + t6 * r3.y),
							      k2 * (t4 * r1.z + t5 * r2.z + t6 * r3.z));
				if (role == 0) {
					fx += f1.x; fy += f1.y; fz += f1.z;
					ed += gg[0] + (gg[1] + (gg[2] + (gg[3] + (gg[4] + gg[5] * cc) * cc) * cc) * cc) * cc;
					a.term_out[a.term_off[2] + idx] = 3.14159265358979f - acosf(fminf(fmaxf(cc, -1.f), 1.f));
				} else if (role == 1) {
					fx += -(1.f + cR1) * f1.x + cR2 * f2.x;
					fy += -(1.f + cR1) * f1.y + cR2 * f2.y;
					fz += -(1.f + cR1) * f1.z + cR2 * f2.z;
				} else if (role == 2) {
					fx += cR1 * f1.x - (1.f + cR2) * f2.x;
					fy += cR1 * f1.y - (1.f + cR2) * f2.y;
					fz += cR1 * f1.z - (1.f + cR2) * f2.z;
				} else {
					fx += f2.x; fy += f2.y; fz += f2.z;
				}
			}
		}
	}
#pragma unroll
	for (int o = 1; o < BOND_LPA; o <<= 1) {
		fx += __shfl_xor_sync(0xffffffffu, fx, o);
		fy += __shfl_xor_sync(0xffffffffu, fy, o);
		fz += __shfl_xor_sync(0xffffffffu, fz, o);
	}
	if (s < n && sub == 0) {
		if (a.accumulate) {
			if (fx != 0.f || fy != 0.f || fz != 0.f) {
				float4 f = a.frc[s];
				f.x += fx; f.y += fy; f.z += fz;
				a.frc[s] = f;
			}
		} else {
			a.frc[s] = make_float4(fx, fy, fz, 0.f);
		}
	}
	// the bond slot takes energy, pot_P and pot_P_bond; angles and torsions
	// their energy (kinds not pending add zero to field 0 of slot 0)
	float v[15] = {eb, w[0], w[1], w[2], w[3], w[4], w[5], w[0], w[1], w[2], w[3], w[4], w[5], ea, ed};
	int fld[15];
	fld[0] = a.fld0[0] + SLOT_EPOT0;
#pragma unroll
	for (int k = 0; k < 6; k++) {
		fld[1 + k] = a.fld0[0] + SLOT_POTP + k;
		fld[7 + k] = a.fld0[0] + SLOT_POTPB + k;
	}
	fld[13] = a.fld0[1] + SLOT_EPOT0;
	fld[14] = a.fld0[2] + SLOT_EPOT0;
	block_to_slot<15>(v, fld, a.slots, 0.f, -1);
}

template <class T>
static int upload(sepdev *d, T **dst, const T *src, size_t count)
{
	if (*dst) { cudaFree(*dst); *dst = NULL; }
	CK(cudaMalloc((void **)dst, sizeof(T) * (count ? count : 1)));
	if (count) CK(cudaMemcpyAsync(*dst, src, sizeof(T) * count, cudaMemcpyHostToDevice, d->st));
	return SEPDEV_OK;
}

extern "C" int sepdev_set_topology(sepdev *d, int nb, const unsigned *blist, int na,
				   const unsigned *alist, int nd, const unsigned *dlist)
{
	const long n = d->n;
	uint4 *hb = (uint4 *)malloc(sizeof(uint4) * (nb ? nb : 1));
	uint4 *ha = (uint4 *)malloc(sizeof(uint4) * (na ? na : 1));
	uint4 *hd = (uint4 *)malloc(sizeof(uint4) * (nd ? nd : 1));
	int *ht = (int *)malloc(sizeof(int) * (nd ? nd : 1));
	int *cnt = (int *)calloc(n + 1, sizeof(int));
	const long nterm = 2L * nb + 3L * na + 4L * nd;
	int *inc = (int *)malloc(sizeof(int) * (nterm ? nterm : 1));
	int rc = SEPDEV_OK;
	if (!hb || !ha || !hd || !ht || !cnt || !inc) { rc = SEPDEV_ENOMEM; goto out; }
	for (int t = 0; t < nb; t++) {
		hb[t] = make_uint4(blist[3 * t], blist[3 * t + 1], blist[3 * t + 2], 0u);
		for (int r = 0; r < 2; r++) {
			unsigned a = blist[3 * t + r];
			if (a >= (unsigned)n) { rc = SEPDEV_EINVAL; goto out; }
			cnt[a + 1]++;
		}
	}
	for (int t = 0; t < na; t++) {
		ha[t] = make_uint4(alist[4 * t], alist[4 * t + 1], alist[4 * t + 2], alist[4 * t + 3]);
		for (int r = 0; r < 3; r++) {
			unsigned a = alist[4 * t + r];
			if (a >= (unsigned)n) { rc = SEPDEV_EINVAL; goto out; }
			cnt[a + 1]++;
		}
	}
	for (int t = 0; t < nd; t++) {
		hd[t] = make_uint4(dlist[5 * t], dlist[5 * t + 1], dlist[5 * t + 2], dlist[5 * t + 3]);
		ht[t] = (int)dlist[5 * t + 4];
		for (int r = 0; r < 4; r++) {
			unsigned a = dlist[5 * t + r];
			if (a >= (unsigned)n) { rc = SEPDEV_EINVAL; goto out; }
			cnt[a + 1]++;
		}
	}
	for (long i = 0; i < n; i++) cnt[i + 1] += cnt[i];
	{
		int *fill = (int *)malloc(sizeof(int) * n);
		if (!fill) { rc = SEPDEV_ENOMEM; goto out; }
		memcpy(fill, cnt, sizeof(int) * n);
		for (int t = 0; t < nb; t++)
			for (int r = 0; r < 2; r++) inc[fill[blist[3 * t + r]]++] = (int)ENC(TERM_BOND, r, t);
		for (int t = 0; t < na; t++)
			for (int r = 0; r < 3; r++) inc[fill[alist[4 * t + r]]++] = (int)ENC(TERM_ANGLE, r, t);
		for (int t = 0; t < nd; t++)
			for (int r = 0; r < 4; r++) inc[fill[dlist[5 * t + r]]++] = (int)ENC(TERM_DIHED, r, t);
		free(fill);
	}
	if ((rc = upload(d, &d->bonds, hb, nb)) || (rc = upload(d, &d->angles, ha, na)) ||
	    (rc = upload(d, &d->diheds_abcd, hd, nd)) || (rc = upload(d, &d->dihed_type, ht, nd)) ||
	    (rc = upload(d, &d->inc_start, cnt, n + 1)) || (rc = upload(d, &d->inc_term, inc, nterm)))
		goto out;
	if (d->term_out) cudaFree(d->term_out);
	d->term_out = NULL;
	if (cudaMalloc((void **)&d->term_out, sizeof(float) * ((size_t)nb + na + nd + 1)) != cudaSuccess) {
		rc = SEPDEV_ENOMEM;
		goto out;
	}
	cudaMemsetAsync(d->term_out, 0, sizeof(float) * ((size_t)nb + na + nd + 1), d->st);
	d->nbond = nb; d->nangle = na; d->ndihed = nd;
	if (cudaStreamSynchronize(d->st) != cudaSuccess) rc = SEPDEV_ECUDA;
out:
	free(hb); free(ha); free(hd); free(ht); free(cnt); free(inc);
	return rc;
}

extern "C" int sepdev_bonded(sepdev *d, const sepdev_bterm *t, int nt, int accumulate)
{
	if (!d->inc_start || nt < 1 || nt > 3) return SEPDEV_EINVAL;
	BondArgs a;
	memset(&a, 0, sizeof a);
	a.pos = d->pos[d->cur]; a.xlo = d->xlo; a.frc = d->frc;
	a.gid = d->gid; a.inv = d->inv;
	a.inc_start = d->inc_start; a.inc_term = d->inc_term;
	a.bonds = d->bonds; a.angles = d->angles; a.diheds = d->diheds_abcd; a.dtype = d->dihed_type;
	a.term_out = d->term_out;
	a.term_off[0] = 0; a.term_off[1] = d->nbond; a.term_off[2] = (long)d->nbond + d->nangle;
	for (int k = 0; k < 3; k++) a.fs[k] = d->fscale[k];
	for (int q = 0; q < nt; q++) {
		const int k = t[q].kind;
		if (k < 0 || k > 2 || a.has[k] || t[q].slot < 0 || t[q].slot >= d->nslots) return SEPDEV_EINVAL;
		a.has[k] = 1;
		a.type[k] = t[q].type;
		a.fld0[k] = t[q].slot * SLOT_FIELDS;
		if (k == TERM_BOND) {
			a.bl0 = (float)t[q].p0; a.bk = (float)t[q].p1;
		} else if (k == TERM_ANGLE) {
			a.cossq = t[q].cossq;
			a.ap0 = t[q].cossq ? (float)cos(3.14159265358979 - t[q].p0) : (float)t[q].p0;
			a.ak = (float)t[q].p1;
		} else {
			for (int g = 0; g < 6; g++) a.g[g] = (float)t[q].g[g];
		}
	}
	a.accumulate = accumulate;
	a.slots = d->slots;
	k_bonded<<<grid_for(d->n * BOND_LPA, 256), 256, 0, d->st>>>(d->n, a);
	CKL(d);
	return SEPDEV_OK;
}

extern "C" int sepdev_term_values(sepdev *d, int kind, double *out)
{
	const long off = kind == 0 ? 0 : (kind == 1 ? d->nbond : (long)d->nbond + d->nangle);
	const long cnt = kind == 0 ? d->nbond : (kind == 1 ? d->nangle : d->ndihed);
	if (cnt == 0 || !d->term_out) return SEPDEV_OK;
	float *h = (float *)malloc(sizeof(float) * cnt);
	if (!h) return SEPDEV_ENOMEM;
	cudaError_t e = cudaMemcpyAsync(h, d->term_out + off, sizeof(float) * cnt, cudaMemcpyDeviceToHost, d->st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
	if (e != cudaSuccess) { free(h); sepdev_set_error("term_values", e); return SEPDEV_ECUDA; }
	for (long t = 0; t < cnt; t++) out[t] = h[t];
	free(h);
	return SEPDEV_OK;
}
