// dev_pair.cu - pair forces, Nose-Hoover friction and leap-frog.
//
// Reference semantics restated here:
//   pair force      source/sepprfrc.c:94-224 (generic callback) and :782-923
//                   (inlined LJ); per pair ft(r^2), f = ft r, U, f_k r_kk
//   SF Coulomb      source/sepcoulomb.c:96-160
//   Nose-Hoover     source/sepintgr.c:149-168 (alpha computed by the caller)
//   leap-frog       source/sepintgr.c:18-88
//
// GB300 design:
//   * FULL neighbour list: each particle sums all its pair forces itself, so
//     no atomics touch the force array; energies and virials are halved.
//   * one lane per particle walks its list in warp tiles: the lanes of a
//     warp read the same group of four entries of their 32 lists with one
//     coalesced 512-byte load (the layout is nl_index, dev_common.cuh).
//   * j positions are 16-byte int4 gathers through the read-only path;
//     separations are int32 differences of fixed-point high words
//     (minimum image by wrap-around) converted to FP32.
//   * the fused step kernel computes the force of particle i from the
//     positions of step t (buffer cur) and immediately integrates i into
//     buffer cur^1, so one launch and one pass over the particle state per
//     MD step suffice.
#include <math.h>
#include <string.h>
#include "dev_common.cuh"

#include "dev_pair.cuh"
#include "dev_batch.cuh"

enum { VAR_SINGLE = 0, VAR_GENERAL = 1, VAR_GENERAL_COUL = 2 };

__device__ __forceinline__ void lj_eval(float r2, float sig2, float eps48, float eps4, float awh,
					float aw, float ushift, float &ft, float &u)
{
	const float s2 = sig2 * fast_rcp(r2);
	const float s6 = s2 * s2 * s2;
	ft = eps48 * s6 * (s6 - awh) * s2;   // the reference multiplies by sigma^2/r^2
	u = eps4 * s6 * (s6 - aw) + ushift;
}

__device__ __forceinline__ void tab_eval(const float2 *__restrict__ t, int nt, float r2min,
					 float idr2, float r2, float &ft, float &u)
{
	float xk = (r2 - r2min) * idr2;
	xk = fminf(fmaxf(xk, 0.f), (float)(nt - 1) - 1e-3f);
	const int k = (int)xk;
	const float w = xk - (float)k;
	const float2 a = __ldg(&t[k]), b = __ldg(&t[k + 1]);
	ft = a.x + w * (b.x - a.x);
	u = a.y + w * (b.y - a.y);
}

// The eight kinetic fields of integrate_s into positions at..at+7 of a
// reduction (slot fields relative to the reduction's base slot by off).
template <int NQ>
__device__ __forceinline__ void kin_fields(const long long (&kq)[8], int off, int at,
					   long long (&q)[NQ], int (&fld)[NQ])
{
	q[at] = kq[0]; fld[at] = off + SLOT_EKIN;
#pragma unroll
	for (int k = 0; k < 6; k++) { q[at + 1 + k] = kq[1 + k]; fld[at + 1 + k] = off + SLOT_KINP + k; }
	q[at + 7] = kq[7]; fld[at + 7] = off + SLOT_SUMV2;
}

// Integrate particle i (leap-frog, optional friction) and return its kinetic
// contributions; F is the total force before friction.  fs, shi, slo: the
// box-dependent scales (L/2^32 and dt*2^64/L split in two floats).
// The velocity increment a dt and the half-step velocity v(t) = v - a dt/2
// are float-float, and the kinetic terms leave as exact fixed point:
// kq = {sum_k m v_k^2, m v_x v_x, m v_x v_y, m v_x v_z, m v_y v_y, m v_y v_z,
// m v_z v_z} at v(t), and kq[7] = m |v(t + dt/2)|^2 (the next thermostat
// update's sum).
__device__ __forceinline__ void integrate_s(long i, float fx, float fy, float fz, float ei,
					    const int4 pi, const PairArgs &a, const float (&fs)[3],
					    const float (&shi)[3], const float (&slo)[3], float alpha,
					    int4 *pos_out, long long (&kq)[8], float &d2)
{
	// the per-particle state is read and written once per step: streaming
	// accesses keep it from displacing the neighbours' positions in L1
	float4 vh = __ldcs(&a.vhi[i]), vl = __ldcs(&a.vlo[i]);
	const uint4 lo = __ldcs(&a.xlo[i]);
	const float m = vh.w, im = vl.w;
	// every product and sum below is an explicit rounding, so the compiler
	// cannot contract differently in the kernels that share this code
	if (a.nh) {
		const float am = __fmul_rn(alpha, m);
		fx = __fmaf_rn(-am, vh.x, fx); fy = __fmaf_rn(-am, vh.y, fy); fz = __fmaf_rn(-am, vh.z, fz);
	}
	__stcs(&a.frc[i], make_float4(fx, fy, fz, ei));
	// a dt with dt carried to ~48 bits, as a float-float (qh, ql)
	const float ax = __fmul_rn(fx, im), ay = __fmul_rn(fy, im), az = __fmul_rn(fz, im);
	const float qhx = __fmul_rn(ax, a.dt), qhy = __fmul_rn(ay, a.dt), qhz = __fmul_rn(az, a.dt);
	const float qlx = __fadd_rn(__fmaf_rn(ax, a.dt, -qhx), __fmul_rn(ax, a.dt_lo));
	const float qly = __fadd_rn(__fmaf_rn(ay, a.dt, -qhy), __fmul_rn(ay, a.dt_lo));
	const float qlz = __fadd_rn(__fmaf_rn(az, a.dt, -qhz), __fmul_rn(az, a.dt_lo));
	ff_add(vh.x, vl.x, qhx); vl.x += qlx;
	ff_add(vh.y, vl.y, qhy); vl.y += qly;
	ff_add(vh.z, vl.z, qhz); vl.z += qlz;
	// v(t) = v(t + dt/2) - q/2 (halving is exact)
	float th[3], tl[3];
	{
		const float vv[3][2] = {{vh.x, vl.x}, {vh.y, vl.y}, {vh.z, vl.z}};
		const float qq[3][2] = {{qhx, qlx}, {qhy, qly}, {qhz, qlz}};
#pragma unroll
		for (int k = 0; k < 3; k++) {
			th[k] = vv[k][0];
			tl[k] = vv[k][1];
			ff_add(th[k], tl[k], -0.5f * qq[k][0]);
			tl[k] = __fadd_rn(tl[k], -0.5f * qq[k][1]);
		}
	}
	{
		const int ka[6] = {0, 0, 0, 1, 1, 2}, kb[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
		for (int c = 0; c < 6; c++) {
			float h, l;
			ff_mprod(m, th[ka[c]], tl[ka[c]], th[kb[c]], tl[kb[c]], h, l);
			kq[1 + c] = to_fx2(h, l);
		}
		kq[0] = kq[1] + kq[4] + kq[6];
		float h0, l0, h1, l1, h2, l2;
		ff_mprod(m, vh.x, vl.x, vh.x, vl.x, h0, l0);
		ff_mprod(m, vh.y, vl.y, vh.y, vl.y, h1, l1);
		ff_mprod(m, vh.z, vl.z, vh.z, vl.z, h2, l2);
		kq[7] = to_fx(h0) + to_fx(h1) + to_fx(h2) + to_fx(__fadd_rn(__fadd_rn(l0, l1), l2));
	}
	const long long ix = ff_mul_fix(vh.x, vl.x, shi[0], slo[0]);
	const long long iy = ff_mul_fix(vh.y, vl.y, shi[1], slo[1]);
	const long long iz = ff_mul_fix(vh.z, vl.z, shi[2], slo[2]);
	const unsigned long long X0 = ((unsigned long long)(unsigned)pi.x << 32) | lo.x;
	const unsigned long long Y0 = ((unsigned long long)(unsigned)pi.y << 32) | lo.y;
	const unsigned long long Z0 = ((unsigned long long)(unsigned)pi.z << 32) | lo.z;
	const unsigned long long X1 = X0 + (unsigned long long)ix;
	const unsigned long long Y1 = Y0 + (unsigned long long)iy;
	const unsigned long long Z1 = Z0 + (unsigned long long)iz;
	const int cx = (ix > 0 && X1 < X0) ? 1 : ((ix < 0 && X1 > X0) ? -1 : 0);
	const int cy = (iy > 0 && Y1 < Y0) ? 1 : ((iy < 0 && Y1 > Y0) ? -1 : 0);
	const int cz = (iz > 0 && Z1 < Z0) ? 1 : ((iz < 0 && Z1 > Z0) ? -1 : 0);
	if (cx | cy | cz) {
		int4 c = a.cross[i];
		c.x += cx; c.y += cy; c.z += cz;
		a.cross[i] = c;
	}
	const int4 po = make_int4((int)(unsigned)(X1 >> 32), (int)(unsigned)(Y1 >> 32),
				  (int)(unsigned)(Z1 >> 32), pi.w);
	pos_out[i] = po;
	__stcs(&a.xlo[i], make_uint4((unsigned)X1, (unsigned)Y1, (unsigned)Z1, 0u));
	__stcs(&a.vhi[i], vh);
	__stcs(&a.vlo[i], vl);
	const int4 xn = __ldcs(&a.xn[i]);
	const float dx = sep_hi(po.x, xn.x, fs[0]);
	const float dy = sep_hi(po.y, xn.y, fs[1]);
	const float dz = sep_hi(po.z, xn.z, fs[2]);
	d2 = dx * dx + dy * dy + dz * dz;
}

__device__ __forceinline__ void integrate(long i, float fx, float fy, float fz, float ei,
					  const int4 pi, const PairArgs &a, float alpha, int4 *pos_out,
					  long long (&kq)[8], float &d2)
{
	integrate_s(i, fx, fy, fz, ei, pi, a, a.fs, a.shi, a.slo, alpha, pos_out, kq, d2);
}

// MOLV: also the molecular virial of the pass.  For each pair of atoms in
// different molecules (both molecule indices set) the pair force f adds
// f (x) R_ij, R_ij the minimum image of the two molecules' centres of mass
// at this pass, and f (x) n_ij, n_ij the periodic image (-1, 0, 1 per axis)
// that minimum image takes; both nine components, halved for the full list,
// into fields 0-8 and 9-17 of slot a.mslot.  f is also added to the atom's
// intermolecular force.
template <int VAR, bool FUSED, bool MOLV = false>
__global__ void __launch_bounds__(256) k_pair(long n, PairArgs a)
{
	constexpr int NCH = VAR == VAR_SINGLE ? 1 : 4;
	extern __shared__ sepdev_pot spot[];
	if (FUSED) step_decide_entry(a.dec);
	if (a.flags && (a.flags[0] & 1u)) {           // list overflow: leave the state untouched
		if (FUSED) {
			step_decide_skip(a.dec);
			step_take_skip(a.take);
		}
		return;
	}
	int ntypes = 1;
	if (VAR != VAR_SINGLE) {
		ntypes = a.ps->ntypes;
		for (int k = threadIdx.x; k < ntypes * ntypes; k += blockDim.x) spot[k] = a.ps->pot[k];
		__syncthreads();
	}
	const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
	const bool act = i < n;
	float fx = 0.f, fy = 0.f, fz = 0.f;
	float e[NCH];
#pragma unroll
	for (int c = 0; c < NCH; c++) e[c] = 0.f;
	float ec = 0.f;
	float w0 = 0.f, w1 = 0.f, w2 = 0.f, w3 = 0.f, w4 = 0.f, w5 = 0.f;
	float wm[18];
#pragma unroll
	for (int k = 0; k < 18; k++) wm[k] = 0.f;
	float gix = 0.f, giy = 0.f, giz = 0.f;
	int mi = -1;
	int4 ci = make_int4(0, 0, 0, 0);
	int4 pi = make_int4(0, 0, 0, 0);
	if (act) {
		pi = a.pos[i];
		if (MOLV) {
			mi = a.mol[i];
			if (mi >= 0) ci = a.mcm[mi];
		}
		const int cnt = a.ncnt[i];
		const int *base = a.nl + nl_index(i, 0, a.maxnb);
		float qi = 0.f;
		bool coul_i = false;
		if (VAR == VAR_GENERAL_COUL) {
			qi = a.charge[i];
			coul_i = fabsf(qi) >= 2.220446049250313e-16f;
		}
		const float sx = a.fs[0], sy = a.fs[1], sz = a.fs[2];
#pragma unroll 4
		for (int k = 0; k < cnt; k++) {
			const int j = __ldg(base + (k >> 2) * 128 + (k & 3));
			const int4 pj = __ldg(&a.pos[j]);
			const float dx = sep_hi(pi.x, pj.x, sx);
			const float dy = sep_hi(pi.y, pj.y, sy);
			const float dz = sep_hi(pi.z, pj.z, sz);
			const float r2 = dx * dx + dy * dy + dz * dz;
			float ft = 0.f;
			if (VAR == VAR_SINGLE) {
				if (r2 < a.rc2) {
					float u;
					lj_eval(r2, a.sig2, a.eps48, a.eps4, a.awh, a.aw, a.ushift, ft, u);
					e[0] += u;
				}
			} else {
				const sepdev_pot &pp = spot[pi.w * ntypes + pj.w];
				if (pp.kind != SEPDEV_POT_OFF && r2 < pp.rc2) {
					float u;
					if (pp.kind == SEPDEV_POT_LJ)
						lj_eval(r2, pp.sig2, pp.eps48, pp.eps4, pp.awh, pp.aw, pp.ushift, ft, u);
					else
						tab_eval(a.tab[pp.table], a.tab_n[pp.table], a.tab_r2min[pp.table],
							 a.tab_idr2[pp.table], r2, ft, u);
#pragma unroll
					for (int c = 0; c < NCH; c++) e[c] += (pp.chan == c) ? u : 0.f;
				}
				if (VAR == VAR_GENERAL_COUL && coul_i && r2 < a.ps->coul_rc2) {
					const float qq = qi * __ldg(&a.charge[j]);
					const float ir = rsqrtf(r2), r = r2 * ir, ir2 = ir * ir;
					ft += qq * (ir2 - a.ps->coul_irc2) * ir;
					ec += qq * (ir + (r - a.ps->coul_rc) * a.ps->coul_irc2 - a.ps->coul_irc);
				}
			}
			const float gx = ft * dx, gy = ft * dy, gz = ft * dz;
			fx += gx; fy += gy; fz += gz;
			w0 += gx * dx; w1 += gx * dy; w2 += gx * dz;
			w3 += gy * dy; w4 += gy * dz; w5 += gz * dz;
			if (MOLV && mi >= 0) {
				const int mj = __ldg(&a.mol[j]);
				if (mj >= 0 && mj != mi) {
					const int4 cj = __ldg(&a.mcm[mj]);
					const unsigned hi[3] = {(unsigned)ci.x, (unsigned)ci.y, (unsigned)ci.z};
					const unsigned hj[3] = {(unsigned)cj.x, (unsigned)cj.y, (unsigned)cj.z};
					const float sc[3] = {sx, sy, sz}, g3[3] = {gx, gy, gz};
					float R[3], nim[3];
#pragma unroll
					for (int q = 0; q < 3; q++) {
						const int dI = (int)(hi[q] - hj[q]);
						R[q] = (float)dI * sc[q];
						nim[q] = (float)((((long long)hi[q] - (long long)hj[q]) - dI) >> 32);
					}
#pragma unroll
					for (int p = 0; p < 3; p++)
#pragma unroll
						for (int q = 0; q < 3; q++) {
							wm[3 * p + q] += g3[p] * R[q];
							wm[9 + 3 * p + q] += g3[p] * nim[q];
						}
					gix += gx; giy += gy; giz += gz;
				}
			}
		}
		if (MOLV && mi >= 0) {
			float4 fo = a.finter[a.gid[i]];
			fo.x += gix; fo.y += giy; fo.z += giz;
			a.finter[a.gid[i]] = fo;
		}
	}
	float etot = ec;
#pragma unroll
	for (int c = 0; c < NCH; c++) etot += e[c];
	long long kq[8] = {0, 0, 0, 0, 0, 0, 0, 0};
	float d2 = 0.f;
	if (act) {
		if (a.accumulate) {
			const float4 fo = a.frc[i];
			fx += fo.x; fy += fo.y; fz += fo.z;
		}
		if (FUSED) {
			const float alpha = a.alpha_dev ? (float)*a.alpha_dev : a.alpha;
			integrate(i, fx, fy, fz, 0.5f * etot, pi, a, alpha, a.pos_out, kq, d2);
		} else {
			a.frc[i] = make_float4(fx, fy, fz, 0.5f * etot);
		}
	}
	// reductions: pair terms (halved for the full list) into pslot, kinetic into lslot
	long long *ps = a.slots + (long)a.pslot * SLOT_FIELDS;
	constexpr int NM = MOLV ? 18 : 0;
	const int moff = (a.mslot - a.pslot) * SLOT_FIELDS;
	if (!FUSED) {
		float v[NCH + 7 + NM];
		int fld[NCH + 7 + NM];
#pragma unroll
		for (int c = 0; c < NCH; c++) { v[c] = 0.5f * e[c]; fld[c] = SLOT_EPOT0 + c; }
		v[NCH] = 0.5f * ec; fld[NCH] = SLOT_ECOUL;
		v[NCH + 1] = 0.5f * w0; v[NCH + 2] = 0.5f * w1; v[NCH + 3] = 0.5f * w2;
		v[NCH + 4] = 0.5f * w3; v[NCH + 5] = 0.5f * w4; v[NCH + 6] = 0.5f * w5;
#pragma unroll
		for (int k = 0; k < 6; k++) fld[NCH + 1 + k] = SLOT_POTP + k;
#pragma unroll
		for (int k = 0; k < NM; k++) { v[NCH + 7 + k] = 0.5f * wm[k]; fld[NCH + 7 + k] = moff + k; }
		block_to_slot<NCH + 7 + NM>(v, fld, ps, 0.f, -1);
	} else {
		long long *ls = a.slots + (long)a.lslot * SLOT_FIELDS;
		const long long off = ls - ps;
		long long q[NCH + 15 + NM];
		int fld[NCH + 15 + NM];
#pragma unroll
		for (int c = 0; c < NCH; c++) { q[c] = to_fx(0.5f * e[c]); fld[c] = SLOT_EPOT0 + c; }
		q[NCH] = to_fx(0.5f * ec); fld[NCH] = SLOT_ECOUL;
		q[NCH + 1] = to_fx(0.5f * w0); q[NCH + 2] = to_fx(0.5f * w1); q[NCH + 3] = to_fx(0.5f * w2);
		q[NCH + 4] = to_fx(0.5f * w3); q[NCH + 5] = to_fx(0.5f * w4); q[NCH + 6] = to_fx(0.5f * w5);
#pragma unroll
		for (int k = 0; k < 6; k++) fld[NCH + 1 + k] = SLOT_POTP + k;
		kin_fields<NCH + 15 + NM>(kq, (int)off, NCH + 7, q, fld);
#pragma unroll
		for (int k = 0; k < NM; k++) { q[NCH + 15 + k] = to_fx(0.5f * wm[k]); fld[NCH + 15 + k] = moff + k; }
		block_to_slot_fx<NCH + 15 + NM>(q, fld, ps, d2, (int)off + SLOT_MAXD2);
		step_decide_exit(a.dec);
		step_take_exit(a.take);
	}
}

// Sums of a cubic box's pair loop back to real units: forces times u,
// virial times u^2, each with both halves of the float pair.
__device__ __forceinline__ void lj_rescale(const LjScale &c, float &fx, float &fy, float &fz, float (&w)[6])
{
	fx = __fmaf_rn(fx, c.ul, __fmul_rn(fx, c.uh));
	fy = __fmaf_rn(fy, c.ul, __fmul_rn(fy, c.uh));
	fz = __fmaf_rn(fz, c.ul, __fmul_rn(fz, c.uh));
#pragma unroll
	for (int k = 0; k < 6; k++) w[k] = __fmaf_rn(w[k], c.u2l, __fmul_rn(w[k], c.u2h));
}

// Fast path for one Lennard-Jones potential on all pairs (the plain-LJ
// workload).  A lane owns one particle and consumes its neighbour list in
// batches of eight: two 16-byte loads bring the next eight indices (the
// following batch is already in flight while the current one is computed),
// then eight independent position gathers, then branch-free pair maths with
// the cut-off as a mask.  For a cubic box the box scale is folded out of the
// pair loop: separations stay in fixed-point units (L/2^32) and the
// per-particle sums are rescaled once.
// OBS: accumulate energy, hit count and virial (skipped on steps whose
// sepret nobody reads).
// sig2 = s2h + s2l as a float pair (s2l = 0 where the scale is exact).
// A group of four list entries: read once, so it is not kept in L1, where
// the neighbours' positions need the room.
__device__ __forceinline__ int4 ld_list(const int4 *p)
{
	int4 r;
	asm volatile("ld.global.nc.L1::no_allocate.v4.s32 {%0, %1, %2, %3}, [%4];"
		     : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w) : "l"(p));
	return r;
}

// TEAM lanes share a particle: lane h of the team takes the list's groups
// of four h, h + TEAM, h + 2 TEAM, ...; each lane gathers G groups per
// iteration.  G only changes how many loads are in flight, not the order of
// the sums; TEAM does change it (the partial sums are added afterwards).
template <bool OBS, bool CUBIC, int TEAM, int G>
__device__ __forceinline__ void lj_pairs(const PairArgs &a, long i, int h, int cnt, const int4 &pi,
					 float sx, float sy, float sz, float rc2, float s2h, float s2l,
					 float &fx, float &fy, float &fz, float &e, float &nin,
					 float (&w)[6])
{
	const float eps48 = a.eps48, eps4 = a.eps4, aw = a.aw, nb48 = -a.eps48 * a.awh;
	auto pair4 = [&](const int4 (&pj)[4]) {
#pragma unroll
		for (int b = 0; b < 4; b++) {
			const float dx = (float)(pi.x - pj[b].x) * sx;
			const float dy = (float)(pi.y - pj[b].y) * sy;
			const float dz = (float)(pi.z - pj[b].z) * sz;
			const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
			const bool in = (r2 < rc2) & (r2 > 0.f);
			// pairs outside the cut-off get s2 = 0, which zeroes their
			// force and energy; the shift is added per hit at the end
			const float rr = fast_rcp(r2);
			const float s2 = in ? __fmaf_rn(s2l, rr, __fmul_rn(s2h, rr)) : 0.f;
			const float s6 = s2 * s2 * s2;
			// 48 eps s6 (s6 - aw/2) s2, the reference's force factor
			const float ft = __fmul_rn(__fmul_rn(s2, s6), __fmaf_rn(eps48, s6, nb48));
			// explicit fused forms: observed and unobserved steps give the
			// same force bits whatever the compiler does with the rest
			fx = __fmaf_rn(ft, dx, fx); fy = __fmaf_rn(ft, dy, fy); fz = __fmaf_rn(ft, dz, fz);
			if (OBS) {
				e = fmaf(eps4 * s6, s6 - aw, e);
				nin += in ? 1.f : 0.f;
				const float gx = ft * dx, gy = ft * dy, gz = ft * dz;
				w[0] = fmaf(gx, dx, w[0]); w[1] = fmaf(gx, dy, w[1]); w[2] = fmaf(gx, dz, w[2]);
				w[3] = fmaf(gy, dy, w[3]); w[4] = fmaf(gy, dz, w[4]); w[5] = fmaf(gz, dz, w[5]);
			}
		}
	};
	const int4 *lp = (const int4 *)(a.nl + nl_index(i, 0, a.maxnb));
	const int nb = (cnt + 3) >> 2;
	// G groups per iteration, the next G groups of indices in flight; the
	// last group is padded with i itself, and a group past the end is i
	// four times: the zero separation masks both
	constexpr int STEP = TEAM * G;
	const int4 self4 = make_int4((int)i, (int)i, (int)i, (int)i);
	int4 jn[G];
#pragma unroll
	for (int q = 0; q < G; q++) jn[q] = h + q * TEAM < nb ? ld_list(lp + (h + q * TEAM) * 32) : self4;
	for (int g0 = h; g0 < nb; g0 += STEP) {
		int4 jc[G];
#pragma unroll
		for (int q = 0; q < G; q++) {
			jc[q] = jn[q];
			const int g = g0 + STEP + q * TEAM;
			jn[q] = g < nb ? ld_list(lp + g * 32) : self4;
		}
		int4 pj[G][4];
#pragma unroll
		for (int q = 0; q < G; q++) {
			pj[q][0] = __ldg(&a.pos[jc[q].x]); pj[q][1] = __ldg(&a.pos[jc[q].y]);
			pj[q][2] = __ldg(&a.pos[jc[q].z]); pj[q][3] = __ldg(&a.pos[jc[q].w]);
		}
#pragma unroll
		for (int q = 0; q < G; q++) pair4(pj[q]);
	}
}

// the partial sums of a team's second lane onto its first (lanes 0-15 of
// the warp hold the particles, lanes 16-31 their second halves)
template <int TEAM>
__device__ __forceinline__ void team_sum(float &fx, float &fy, float &fz, float &e, float &nin,
					 float (&w)[6])
{
	if (TEAM == 1) return;
	const unsigned FULL = 0xffffffffu;
	fx += __shfl_down_sync(FULL, fx, 16); fy += __shfl_down_sync(FULL, fy, 16);
	fz += __shfl_down_sync(FULL, fz, 16); e += __shfl_down_sync(FULL, e, 16);
	nin += __shfl_down_sync(FULL, nin, 16);
#pragma unroll
	for (int k = 0; k < 6; k++) w[k] += __shfl_down_sync(FULL, w[k], 16);
}

// TEAM lanes per particle: a warp holds 32 / TEAM particles; after the
// pair loop the first lane of each team carries the particle on alone.
template <bool FUSED, bool CUBIC, int TEAM, int G>
__global__ void __launch_bounds__(256, 4) k_lj(long n, PairArgs a)
{
	if (FUSED) step_decide_entry(a.dec);
	if (a.flags && (a.flags[0] & 1u)) {
		if (FUSED) {
			step_decide_skip(a.dec);
			step_take_skip(a.take);
		}
		return;
	}
	constexpr int PPW = 32 / TEAM;
	const int lane = threadIdx.x & 31, h = lane / PPW;
	const long i = (blockIdx.x * (long)blockDim.x + threadIdx.x) / 32 * PPW + lane % PPW;
	const bool inrange = i < n;
	const float sx = CUBIC ? 1.f : a.fs[0], sy = CUBIC ? 1.f : a.fs[1], sz = CUBIC ? 1.f : a.fs[2];
	const float rc2 = CUBIC ? a.sc.rc2s : a.rc2;
	const float s2h = CUBIC ? a.sc.s2h : a.sig2, s2l = CUBIC ? a.sc.s2l : 0.f;
	float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f, nin = 0.f;
	float w[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
	int4 pi = make_int4(0, 0, 0, 0);
	const int cnt = inrange ? a.ncnt[i] : 0;
	const bool obs = !FUSED || (!a.skip_obs && step_observed(a.dec));
	if (inrange) {
		pi = a.pos[i];
		if (obs)
			lj_pairs<true, CUBIC, TEAM, G>(a, i, h, cnt, pi, sx, sy, sz, rc2, s2h, s2l, fx, fy, fz, e, nin, w);
		else
			lj_pairs<false, CUBIC, TEAM, G>(a, i, h, cnt, pi, sx, sy, sz, rc2, s2h, s2l, fx, fy, fz, e, nin, w);
	}
	team_sum<TEAM>(fx, fy, fz, e, nin, w);
	const bool act = inrange && h == 0;
	if (!act) {
		fx = fy = fz = e = nin = 0.f;
#pragma unroll
		for (int k = 0; k < 6; k++) w[k] = 0.f;
	}
	e = fmaf(nin, a.ushift, e);
	if (CUBIC) lj_rescale(a.sc, fx, fy, fz, w);
	const float w0 = w[0], w1 = w[1], w2 = w[2], w3 = w[3], w4 = w[4], w5 = w[5];
	long long kq[8] = {0, 0, 0, 0, 0, 0, 0, 0};
	float d2 = 0.f;
	if (act) {
		if (a.accumulate) {
			const float4 fo = a.frc[i];
			fx += fo.x; fy += fo.y; fz += fo.z;
		}
		if (FUSED) {
			const float alpha = a.alpha_dev ? (float)*a.alpha_dev : a.alpha;
			integrate(i, fx, fy, fz, 0.5f * e, pi, a, alpha, a.pos_out, kq, d2);
		} else {
			a.frc[i] = make_float4(fx, fy, fz, 0.5f * e);
		}
	}
	long long *ps = a.slots + (long)a.pslot * SLOT_FIELDS;
	if (!FUSED) {
		const long long q[7] = {to_fx2(0.5f * e, 0.5f * nin * a.ushl), to_fx(0.5f * w0), to_fx(0.5f * w1),
					to_fx(0.5f * w2), to_fx(0.5f * w3), to_fx(0.5f * w4), to_fx(0.5f * w5)};
		const int fld[7] = {SLOT_EPOT0, SLOT_POTP, SLOT_POTP + 1, SLOT_POTP + 2, SLOT_POTP + 3,
				    SLOT_POTP + 4, SLOT_POTP + 5};
		block_to_slot_fx<7>(q, fld, ps, 0.f, -1);
	} else {
		const int off = (int)((long)(a.lslot - a.pslot) * SLOT_FIELDS);
		long long q[15] = {to_fx2(0.5f * e, 0.5f * nin * a.ushl), to_fx(0.5f * w0), to_fx(0.5f * w1),
				   to_fx(0.5f * w2), to_fx(0.5f * w3), to_fx(0.5f * w4), to_fx(0.5f * w5)};
		int fld[15] = {SLOT_EPOT0, SLOT_POTP, SLOT_POTP + 1, SLOT_POTP + 2, SLOT_POTP + 3,
			       SLOT_POTP + 4, SLOT_POTP + 5};
		kin_fields<15>(kq, off, 7, q, fld);
		block_to_slot_fx<15>(q, fld, ps, d2, off + SLOT_MAXD2);
		step_decide_exit(a.dec);
		step_take_exit(a.take);
	}
}

// Standalone leap-frog on the stored forces (in-place position update).
__global__ void __launch_bounds__(256) k_leapfrog(long n, PairArgs a)
{
	const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
	long long kq[8] = {0, 0, 0, 0, 0, 0, 0, 0};
	float d2 = 0.f;
	if (i < n) {
		const float4 f = a.frc[i];
		const float alpha = a.alpha_dev ? (float)*a.alpha_dev : a.alpha;
		integrate(i, f.x, f.y, f.z, f.w, a.pos[i], a, alpha, (int4 *)a.pos, kq, d2);
	}
	long long q[8];
	int fld[8];
	kin_fields<8>(kq, 0, 0, q, fld);
	block_to_slot_fx<8>(q, fld, a.slots + (long)a.lslot * SLOT_FIELDS, d2, SLOT_MAXD2);
}

__global__ void k_friction(long n, float alpha, const float4 *__restrict__ vhi, float4 *frc)
{
	const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
	if (i >= n) return;
	const float4 v = vhi[i];
	float4 f = frc[i];
	const float am = alpha * v.w;
	f.x -= am * v.x; f.y -= am * v.y; f.z -= am * v.z;
	frc[i] = f;
}

// ---- host side -----------------------------------------------------------------

static bool single_variant(const sepdev_pairset *ps)
{
	return ps->ntypes == 1 && !ps->coulomb && ps->pot[0].kind == SEPDEV_POT_LJ &&
	       ps->pot[0].chan == 0;
}

void sepdev_fill_args(sepdev *d, PairArgs &a, const sepdev_pairset *ps, double dt, int nh,
		      double alpha, int accumulate, int pslot, int lslot, int parity)
{
	memset(&a, 0, sizeof a);
	a.pos = d->pos[parity];
	a.pos_out = d->pos[parity ^ 1];
	a.xlo = d->xlo; a.vhi = d->vhi; a.vlo = d->vlo; a.frc = d->frc;
	a.xn = d->xn; a.cross = d->cross;
	a.nl = d->nl; a.ncnt = d->ncnt; a.maxnb = d->maxnb;
	a.charge = d->charge;
	for (int k = 0; k < 3; k++) {
		a.fs[k] = d->fscale[k];
		const double S = dt * 18446744073709551616.0 / d->L[k];
		a.shi[k] = (float)S;
		a.slo[k] = (float)(S - (double)a.shi[k]);
	}
	a.ps = d->d_ps;
	if (ps) {
		const sepdev_pot &p0 = ps->pot[0];
		a.rc2 = p0.rc2; a.eps48 = p0.eps48; a.eps4 = p0.eps4; a.sig2 = p0.sig2;
		a.aw = p0.aw; a.awh = p0.awh; a.ushift = p0.ushift; a.ushl = p0.ushl;
		a.sc = lj_scale(d->L[0], (double)p0.sig2, (double)p0.rc2);
	}
	for (int t = 0; t < SEPDEV_MAXTAB; t++) {
		a.tab[t] = d->tab[t]; a.tab_n[t] = d->tab_n[t];
		a.tab_r2min[t] = d->tab_r2min[t]; a.tab_idr2[t] = d->tab_idr2[t];
	}
	a.dt = (float)dt;
	a.dt_lo = (float)(dt - (double)a.dt);
	a.alpha = (float)alpha;
	a.nh = nh;
	a.accumulate = accumulate;
	a.slots = d->slots;
	a.pslot = pslot;
	a.lslot = lslot;
	a.flags = NULL;
	a.skip_obs = 0;
	memset(&a.dec, 0, sizeof a.dec);
	memset(&a.take, 0, sizeof a.take);
}

// Batched systems: one fused step (LJ forces, Nose-Hoover friction,
// leap-frog) over every system at once.  A warp belongs to one system and
// takes that system's box scales, thermostat and kernel parameters (its
// entry of wstep: system, first slot, team size, neighbour groups per
// iteration); the arithmetic per particle is the single-system k_lj's
// (cubic form) under the same parameters, and each warp adds its sums to
// its system's accumulator slot with the same exact fixed-point conversion
// as the block reduction there, so a system's results do not depend on the
// batch.
template <bool OBS>
__device__ __forceinline__ void lj_pairs_any(int team, int groups, const PairArgs &a, long i, int h,
					     int cnt, const int4 &pi, const LjScale &sc, float &fx, float &fy,
					     float &fz, float &e, float &nin, float (&w)[6])
{
	if (team == 1) {
		if (groups == 2)
			lj_pairs<OBS, true, 1, 2>(a, i, h, cnt, pi, 1.f, 1.f, 1.f, sc.rc2s, sc.s2h, sc.s2l, fx, fy, fz, e, nin, w);
		else
			lj_pairs<OBS, true, 1, 1>(a, i, h, cnt, pi, 1.f, 1.f, 1.f, sc.rc2s, sc.s2h, sc.s2l, fx, fy, fz, e, nin, w);
	} else {
		if (groups == 2)
			lj_pairs<OBS, true, 2, 2>(a, i, h, cnt, pi, 1.f, 1.f, 1.f, sc.rc2s, sc.s2h, sc.s2l, fx, fy, fz, e, nin, w);
		else
			lj_pairs<OBS, true, 2, 1>(a, i, h, cnt, pi, 1.f, 1.f, 1.f, sc.rc2s, sc.s2h, sc.s2l, fx, fy, fz, e, nin, w);
	}
}

__global__ void __launch_bounds__(256, 4) k_lj_batch(PairArgs a, const BatchSys *sys, const int4 *wstep,
						    int nwarps, const BatchState *bs, const BatchRun *run,
						    long long *slots, BatchDecide dec)
{
	const unsigned FULL = 0xffffffffu;
	if (dec.reset_while && blockIdx.x == 0 && threadIdx.x == 0)
		cudaGraphSetConditional(dec.h_while, 0);
	if (a.flags && (a.flags[0] & 1u)) return;      // list overflow: the decision stops the loop
	const long wg = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
	if (wg >= nwarps) return;                      // whole warps
	const int4 W = wstep[wg];
	const int s = W.x, team = W.z, ppw = 32 / team, lane = threadIdx.x & 31, h = lane / ppw;
	const long i = W.y + lane % ppw;
	const BatchSys S = sys[s];
	const bool inrange = i - S.off < S.n;
	float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f, nin = 0.f;
	float w[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
	int4 pi = make_int4(0, 0, 0, 0);
	const int cnt = inrange ? a.ncnt[i] : 0;
	const bool obs = run->done + 1 >= run->total;
	if (inrange) {
		pi = a.pos[i];
		if (obs) lj_pairs_any<true>(team, W.w, a, i, h, cnt, pi, S.sc, fx, fy, fz, e, nin, w);
		else lj_pairs_any<false>(team, W.w, a, i, h, cnt, pi, S.sc, fx, fy, fz, e, nin, w);
	}
	if (team == 2) team_sum<2>(fx, fy, fz, e, nin, w);
	const bool act = inrange && h == 0;
	if (!act) {
		fx = fy = fz = e = nin = 0.f;
#pragma unroll
		for (int k = 0; k < 6; k++) w[k] = 0.f;
	}
	e = fmaf(nin, a.ushift, e);
	lj_rescale(S.sc, fx, fy, fz, w);
	long long kq[8] = {0, 0, 0, 0, 0, 0, 0, 0};
	float d2 = 0.f;
	if (act) {
		const float fsv[3] = {S.fs, S.fs, S.fs}, shv[3] = {S.shi, S.shi, S.shi}, slv[3] = {S.slo, S.slo, S.slo};
		const float alpha = (float)bs[s].alpha;
		integrate_s(i, fx, fy, fz, 0.5f * e, pi, a, fsv, shv, slv, alpha, a.pos_out, kq, d2);
	}
	long long q[15] = {to_fx2(0.5f * e, 0.5f * nin * a.ushl), to_fx(0.5f * w[0]), to_fx(0.5f * w[1]),
			   to_fx(0.5f * w[2]), to_fx(0.5f * w[3]), to_fx(0.5f * w[4]), to_fx(0.5f * w[5])};
	int fld[15] = {SLOT_EPOT0, SLOT_POTP, SLOT_POTP + 1, SLOT_POTP + 2, SLOT_POTP + 3,
		       SLOT_POTP + 4, SLOT_POTP + 5};
	kin_fields<15>(kq, 0, 7, q, fld);
#pragma unroll
	for (int k = 0; k < 15; k++) q[k] = warp_sum_fx(q[k]);
	const unsigned mx = __reduce_max_sync(FULL, __float_as_uint(d2));
	if ((threadIdx.x & 31) == 0) {
		long long *sl = slots + (long)s * SLOT_FIELDS;
		for (int k = 0; k < 15; k++)
			if (q[k] != 0) atomicAdd((unsigned long long *)&sl[fld[k]], (unsigned long long)q[k]);
		if (mx) atomicMax((unsigned long long *)&sl[SLOT_MAXD2], (unsigned long long)mx);
	}
}

// Batched systems with one Lennard-Jones parameter set per type pair (the
// reference's one sep_force_lj call per type pair, source/sepprfrc.c:743-1000:
// the term of types "ab" acts on pairs of types a and b in either order; the
// energies of the calls add).  Type ids are in pos.w; the parameter sets
// come from a.ps (unscaled) and are scaled to each system's fixed-point
// units per pair.  A type pair without a term has rc2 = 0 and eps = 0.
template <bool OBS>
__device__ __forceinline__ void ljt_pairs(const PairArgs &a, long i, int cnt, const int4 &pi, float iu2,
					  const sepdev_pot *sp, int nt, float &fx, float &fy, float &fz,
					  float &e, float (&w)[6])
{
	const int4 *lp = (const int4 *)(a.nl + nl_index(i, 0, a.maxnb));
	const int nb = (cnt + 3) >> 2;
	const int row = pi.w * nt;
	int4 jn = nb > 0 ? __ldg(lp) : make_int4(0, 0, 0, 0);
	for (int s0 = 0; s0 < nb; s0++) {
		const int4 jc = jn;
		if (s0 + 1 < nb) jn = __ldg(lp + (s0 + 1) * 32);
		const int rem = cnt - 4 * s0;
		const int j[4] = {jc.x, rem > 1 ? jc.y : (int)i, rem > 2 ? jc.z : (int)i,
				  rem > 3 ? jc.w : (int)i};
		int4 pj[4];
#pragma unroll
		for (int b = 0; b < 4; b++) pj[b] = __ldg(&a.pos[j[b]]);
#pragma unroll
		for (int b = 0; b < 4; b++) {
			const sepdev_pot &pp = sp[row + pj[b].w];
			const float dx = (float)(pi.x - pj[b].x), dy = (float)(pi.y - pj[b].y),
				    dz = (float)(pi.z - pj[b].z);
			const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
			const bool in = (b < rem) && (r2 < pp.rc2 * iu2);
			const float s2 = in ? pp.sig2 * iu2 * fast_rcp(r2) : 0.f;
			const float s6 = s2 * s2 * s2;
			const float ft = __fmul_rn(__fmul_rn(s2, s6), __fmaf_rn(pp.eps48, s6, -pp.eps48 * pp.awh));
			fx = __fmaf_rn(ft, dx, fx); fy = __fmaf_rn(ft, dy, fy); fz = __fmaf_rn(ft, dz, fz);
			if (OBS) {
				const float gx = ft * dx, gy = ft * dy, gz = ft * dz;
				e += in ? fmaf(pp.eps4 * s6, s6 - pp.aw, pp.ushift) : 0.f;
				w[0] = fmaf(gx, dx, w[0]); w[1] = fmaf(gx, dy, w[1]); w[2] = fmaf(gx, dz, w[2]);
				w[3] = fmaf(gy, dy, w[3]); w[4] = fmaf(gy, dz, w[4]); w[5] = fmaf(gz, dz, w[5]);
			}
		}
	}
}

__global__ void __launch_bounds__(256, 4) k_lj_batch_typed(PairArgs a, const BatchSys *sys,
							  const int4 *wstep, int nwarps,
							  const BatchState *bs, const BatchRun *run,
							  long long *slots, BatchDecide dec)
{
	const unsigned FULL = 0xffffffffu;
	__shared__ sepdev_pot sp[SEPB_MAXTYPES * SEPB_MAXTYPES];
	const int nt = a.ps->ntypes;
	for (int k = threadIdx.x; k < nt * nt; k += blockDim.x) sp[k] = a.ps->pot[k];
	__syncthreads();
	if (dec.reset_while && blockIdx.x == 0 && threadIdx.x == 0)
		cudaGraphSetConditional(dec.h_while, 0);
	if (a.flags && (a.flags[0] & 1u)) return;      // list overflow: the decision stops the loop
	const long wg = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
	if (wg >= nwarps) return;                      // whole warps (one lane per particle)
	const int4 W = wstep[wg];
	const int s = W.x;
	const long i = W.y + (threadIdx.x & 31);
	const BatchSys S = sys[s];
	const bool act = i - S.off < S.n;
	const float u = S.fs, iu2 = 1.f / (u * u);
	float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
	float w[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
	int4 pi = make_int4(0, 0, 0, 0);
	const int cnt = act ? a.ncnt[i] : 0;
	const bool obs = run->done + 1 >= run->total;
	if (act) {
		pi = a.pos[i];
		if (obs) ljt_pairs<true>(a, i, cnt, pi, iu2, sp, nt, fx, fy, fz, e, w);
		else ljt_pairs<false>(a, i, cnt, pi, iu2, sp, nt, fx, fy, fz, e, w);
	}
	fx *= u; fy *= u; fz *= u;
	const float u2 = u * u;
	for (int k = 0; k < 6; k++) w[k] *= u2;
	long long kq[8] = {0, 0, 0, 0, 0, 0, 0, 0};
	float d2 = 0.f;
	if (act) {
		const float fsv[3] = {S.fs, S.fs, S.fs}, shv[3] = {S.shi, S.shi, S.shi}, slv[3] = {S.slo, S.slo, S.slo};
		const float alpha = (float)bs[s].alpha;
		integrate_s(i, fx, fy, fz, 0.5f * e, pi, a, fsv, shv, slv, alpha, a.pos_out, kq, d2);
	}
	long long q[15] = {to_fx(0.5f * e), to_fx(0.5f * w[0]), to_fx(0.5f * w[1]), to_fx(0.5f * w[2]),
			   to_fx(0.5f * w[3]), to_fx(0.5f * w[4]), to_fx(0.5f * w[5])};
	int fld[15] = {SLOT_EPOT0, SLOT_POTP, SLOT_POTP + 1, SLOT_POTP + 2, SLOT_POTP + 3,
		       SLOT_POTP + 4, SLOT_POTP + 5};
	kin_fields<15>(kq, 0, 7, q, fld);
#pragma unroll
	for (int k = 0; k < 15; k++) q[k] = warp_sum_fx(q[k]);
	const unsigned mx = __reduce_max_sync(FULL, __float_as_uint(d2));
	if ((threadIdx.x & 31) == 0) {
		long long *sl = slots + (long)s * SLOT_FIELDS;
		for (int k = 0; k < 15; k++)
			if (q[k] != 0) atomicAdd((unsigned long long *)&sl[fld[k]], (unsigned long long)q[k]);
		if (mx) atomicMax((unsigned long long *)&sl[SLOT_MAXD2], (unsigned long long)mx);
	}
}

int sepdev_batch_step(sepdev *d, const PairArgs &a, const BatchSys *sys, const int4 *wstep, int nwarps,
		      const BatchState *bs, const BatchRun *run, long long *slots, const BatchDecide &dec,
		      int typed)
{
	if (typed)
		k_lj_batch_typed<<<grid_for((long)nwarps * 32, 256), 256, 0, d->st>>>(a, sys, wstep, nwarps, bs, run,
										   slots, dec);
	else
		k_lj_batch<<<grid_for((long)nwarps * 32, 256), 256, 0, d->st>>>(a, sys, wstep, nwarps, bs, run, slots,
									       dec);
	CKL(d);
	return SEPDEV_OK;
}

int sepdev_upload_pairset(sepdev *d, const sepdev_pairset *ps)
{
	if (d->ps_valid && memcmp(&d->h_ps, ps, sizeof *ps) == 0) return SEPDEV_OK;
	d->h_ps = *ps;
	CK(cudaMemcpyAsync(d->d_ps, &d->h_ps, sizeof(sepdev_pairset), cudaMemcpyHostToDevice, d->st));
	d->ps_valid = 1;
	return SEPDEV_OK;
}

template <bool FUSED>
static void launch_fused(sepdev *d, int var, const PairArgs &a, size_t shm, bool molv)
{
	const int B = 256;
	const int grid = grid_for(d->n, B);
	const bool cubic = d->L[0] == d->L[1] && d->L[1] == d->L[2];
	if (molv) {
		if (var == VAR_GENERAL_COUL)
			k_pair<VAR_GENERAL_COUL, FUSED, true><<<grid, B, shm, d->st>>>(d->n, a);
		else
			k_pair<VAR_GENERAL, FUSED, true><<<grid, B, shm, d->st>>>(d->n, a);
	} else if (var == VAR_SINGLE && cubic) {
		// the team size and neighbour groups of the system's size class
		const int g2 = grid_for(d->n * d->team, B);
		if (d->team == 2) {
			if (d->groups == 2) k_lj<FUSED, true, 2, 2><<<g2, B, 0, d->st>>>(d->n, a);
			else k_lj<FUSED, true, 2, 1><<<g2, B, 0, d->st>>>(d->n, a);
		} else {
			if (d->groups == 2) k_lj<FUSED, true, 1, 2><<<g2, B, 0, d->st>>>(d->n, a);
			else k_lj<FUSED, true, 1, 1><<<g2, B, 0, d->st>>>(d->n, a);
		}
	} else if (var == VAR_SINGLE)
		k_lj<FUSED, false, 1, 2><<<grid, B, 0, d->st>>>(d->n, a);
	else if (var == VAR_GENERAL)
		k_pair<VAR_GENERAL, FUSED><<<grid, B, shm, d->st>>>(d->n, a);
	else
		k_pair<VAR_GENERAL_COUL, FUSED><<<grid, B, shm, d->st>>>(d->n, a);
}

int sepdev_launch_pair(sepdev *d, const sepdev_pairset *ps, PairArgs &a, bool fused)
{
	const int var = single_variant(ps) ? VAR_SINGLE : (ps->coulomb ? VAR_GENERAL_COUL : VAR_GENERAL);
	const size_t shm = sizeof(sepdev_pot) * ps->ntypes * ps->ntypes;
	// the molecular sums of a pass go to the slot named for it (consumed
	// here, so a launch nobody named a slot for carries none)
	const bool molv = d->molvir_on && d->mv_slot >= 0 && d->mv_slot < d->nslots;
	if (molv) {
		// centres of mass at the positions of this pass
		int rc = sepdev_molvir_cm(d, a.pos);
		if (rc) return rc;
		a.mol = d->mol; a.gid = d->gid; a.mcm = d->mv_cm; a.finter = d->mv_finter;
		a.mslot = d->mv_slot;
	}
	d->mv_slot = -1;
	if (fused) launch_fused<true>(d, var, a, shm, molv);
	else launch_fused<false>(d, var, a, shm, molv);
	CKL(d);
	return SEPDEV_OK;
}

extern "C" int sepdev_pair_forces(sepdev *d, const sepdev_pairset *ps, int accumulate, int slot)
{
	if (!d->list_valid || slot < 0 || slot >= d->nslots) return SEPDEV_EINVAL;
	int rc;
	if ((rc = sepdev_list_confirm(d))) return rc;
	if ((rc = sepdev_upload_pairset(d, ps))) return rc;
	PairArgs a;
	sepdev_fill_args(d, a, ps, 0.0, 0, 0.0, accumulate, slot, slot, d->cur);
	return sepdev_launch_pair(d, ps, a, false);
}

// the fused step on a list that may still be unchecked: the kernel skips its
// work (positions, velocities, forces and sums untouched) when the build
// overflowed; the caller reads the flags with the step's sums.  take_n >= 0:
// the kernel's last block also hands slots [0, take_n) and the flags to the
// host (kept on overflow), for the sepdev_slots_take that follows.
static int step_launch_checked(sepdev *d, const sepdev_pairset *ps, int accumulate, double dt, int nh,
			       double alpha, int pair_slot, int lf_slot, int observe, int take_n)
{
	if (!d->list_valid || pair_slot < 0 || pair_slot >= d->nslots || lf_slot < 0 ||
	    lf_slot >= d->nslots || take_n > d->nslots)
		return SEPDEV_EINVAL;
	int rc;
	if ((rc = sepdev_upload_pairset(d, ps))) return rc;
	PairArgs a;
	sepdev_fill_args(d, a, ps, dt, nh, alpha, accumulate, pair_slot, lf_slot, d->cur);
	a.skip_obs = !observe;
	if (d->list_unchecked) a.flags = d->flags;
	if (take_n >= 0) {
		a.take.h = d->hd_slots;
		a.take.hf = d->hd_flags;
		a.take.arrive = d->take_arrive;
		a.take.slots = d->slots;
		a.take.flags = d->flags;
		a.take.nread = take_n;
		a.take.nall = d->nslots;
		a.take.keep = 1;
	}
	if ((rc = sepdev_launch_pair(d, ps, a, true))) return rc;
	d->take_ready = take_n;
	d->cur ^= 1;
	return SEPDEV_OK;
}

extern "C" int sepdev_step_deferred(sepdev *d, const sepdev_pairset *ps, int accumulate, double dt,
				    int nh, double alpha, int pair_slot, int lf_slot, int take_n)
{
	return step_launch_checked(d, ps, accumulate, dt, nh, alpha, pair_slot, lf_slot, 1, take_n);
}

// a deferred step that found the list overflowed did nothing: its buffer
// flip is undone before the step runs again
extern "C" void sepdev_step_retract(sepdev *d)
{
	d->cur ^= 1;
}

extern "C" int sepdev_step_obs(sepdev *d, const sepdev_pairset *ps, int accumulate, double dt,
			       int nh, double alpha, int pair_slot, int lf_slot, int observe)
{
	if (!d->list_valid) return SEPDEV_EINVAL;
	int rc;
	if ((rc = sepdev_list_confirm(d))) return rc;
	return step_launch_checked(d, ps, accumulate, dt, nh, alpha, pair_slot, lf_slot, observe, -1);
}

extern "C" int sepdev_step(sepdev *d, const sepdev_pairset *ps, int accumulate, double dt,
			   int nh, double alpha, int pair_slot, int lf_slot)
{
	return sepdev_step_obs(d, ps, accumulate, dt, nh, alpha, pair_slot, lf_slot, 1);
}

extern "C" int sepdev_leapfrog(sepdev *d, double dt, int nh, double alpha, int slot)
{
	if (slot < 0 || slot >= d->nslots) return SEPDEV_EINVAL;
	PairArgs a;
	sepdev_fill_args(d, a, NULL, dt, nh, alpha, 0, slot, slot, d->cur);
	const int B = 256;
	k_leapfrog<<<grid_for(d->n, B), B, 0, d->st>>>(d->n, a);
	CKL(d);
	return SEPDEV_OK;
}

extern "C" int sepdev_friction(sepdev *d, double alpha)
{
	const int B = 256;
	k_friction<<<grid_for(d->n, B), B, 0, d->st>>>(d->n, (float)alpha, d->vhi, d->frc);
	CKL(d);
	return SEPDEV_OK;
}

extern "C" int sepdev_zero_forces(sepdev *d)
{
	CK(cudaMemsetAsync(d->frc, 0, sizeof(float4) * d->n, d->st));
	return SEPDEV_OK;
}
