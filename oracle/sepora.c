/*
 * sepora.c - CPU ORACLE for the seplib MD-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain FP64 C99 on
 * structure-of-arrays inputs, the algorithms of the reference library's
 * hot path so that the GPU library can be checked against them.  Nothing in
 * the product (seplib_gb300/) links or calls it; only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg do.
 *
 * Parity is pinned two ways: tests/test_oracle_golden.py checks these
 * functions against golden vectors produced by the reference library itself
 * (tests/golden/make_golden.py, which drives oracle/_ref/libsepref.so built
 * from the reference sources by oracle/Makefile), and, where the reference
 * sources are present, directly against that library.
 *
 * Layout: x, v, f are 3*n doubles, particle-major (x[3*i+k]).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORA_BOND 10
#define ORA_ANGLE 10
#define ORA_DIHED 20

/* exclusion rules, see ora_excluded() */
enum { ORA_EXCL_NONE = 0, ORA_EXCL_BONDS = 1, ORA_EXCL_ALLBONDED = 2, ORA_EXCL_SAMEMOL = 3 };

/* minimum image of one separation component; reference include/sepmisc.h:81-85
 * (strict comparisons against L/2) */
static inline double ora_wrap(double d, double L)
{
	if (d > 0.5 * L) return d - L;
	if (d < -0.5 * L) return d + L;
	return d;
}

static inline double ora_sep(const double *x, long i, long j, const double L[3], double d[3])
{
	double r2 = 0.0;
	for (int k = 0; k < 3; k++) {
		d[k] = ora_wrap(x[3 * i + k] - x[3 * j + k], L[k]);
		r2 += d[k] * d[k];
	}
	return r2;
}

/* membership of j in a -1 terminated partner array of length cap;
 * equivalent to the reference's pairwise scan in source/sepprfrc.c:703-733 for
 * the symmetric partner relations the topology reader builds */
static int ora_in_list(const int *lst, int cap, long j)
{
	for (int k = 0; k < cap && lst[k] != -1; k++)
		if (lst[k] == j) return 1;
	return 0;
}

/*
 * Exclusion predicate.
 *  ORA_EXCL_BONDS     - sep_bond_share only (source/sepprfrc.c:703-711), used by
 *                       the brute pair force and the O(N^2) list for SEP_EXCL_BONDED
 *                       (source/sepprfrc.c:35, :317)
 *  ORA_EXCL_ALLBONDED - sep_bonded = bond + angle + dihedral partners
 *                       (source/sepprfrc.c:736-740), used by the linked-cell list
 *                       (:582) and by the brute SF Coulomb (source/sepcoulomb.c:39)
 *  ORA_EXCL_SAMEMOL   - same molindex and not -1 (source/sepprfrc.c:38-41, :666)
 */
int ora_excluded(int mode, long i, long j, const int *molindex,
		 const int *bond, const int *angle, const int *dihed)
{
	switch (mode) {
	case ORA_EXCL_BONDS:
		return ora_in_list(bond + ORA_BOND * i, ORA_BOND, j) ||
		       ora_in_list(bond + ORA_BOND * j, ORA_BOND, i);
	case ORA_EXCL_ALLBONDED:
		return ora_in_list(bond + ORA_BOND * i, ORA_BOND, j) ||
		       ora_in_list(angle + ORA_ANGLE * i, ORA_ANGLE, j) ||
		       ora_in_list(dihed + ORA_DIHED * i, ORA_DIHED, j) ||
		       ora_in_list(bond + ORA_BOND * j, ORA_BOND, i) ||
		       ora_in_list(angle + ORA_ANGLE * j, ORA_ANGLE, i) ||
		       ora_in_list(dihed + ORA_DIHED * j, ORA_DIHED, i);
	case ORA_EXCL_SAMEMOL:
		return molindex[i] != -1 && molindex[i] == molindex[j];
	default:
		return 0;
	}
}

/*
 * All unordered pairs (i < j) closer than rlist under the minimum image,
 * O(N^2) in FP64.  Restates the brute-force list of source/sepprfrc.c:306-343
 * (criterion r^2 < (cf+skin)^2).  Returns the number of pairs (the array is
 * filled up to maxpairs).
 */
long ora_pairs_brute(long n, const double *x, const double L[3], double rlist,
		     int excl, const int *molindex, const int *bond,
		     const int *angle, const int *dihed, int *pairs, long maxpairs)
{
	const double rl2 = rlist * rlist;
	long np = 0;
	double d[3];
	for (long i = 0; i < n - 1; i++)
		for (long j = i + 1; j < n; j++) {
			if (excl && ora_excluded(excl, i, j, molindex, bond, angle, dihed))
				continue;
			if (ora_sep(x, i, j, L, d) < rl2) {
				if (np < maxpairs) { pairs[2 * np] = (int)i; pairs[2 * np + 1] = (int)j; }
				np++;
			}
		}
	return np;
}

/* number of cells along an edge: floor(L/(cf+delta)) (source/sepmisc.c sep_nsubbox,
 * called with delta = 0.25 by sep_sys_setup, source/sepinit.c:249-276) */
int ora_nsubbox(double cf, double delta, double L)
{
	return (int)floor(L / (cf + delta));
}

/*
 * Half neighbour list from a linked-cell list, as the reference builds it
 * (source/sepprfrc.c:394-415 cell list, :419-513 list build):
 *  - cell of a particle: (int)(x/lsub) per axis, lsub = L/nsub fixed at setup;
 *  - head/next linked cells, filled in particle order so a cell is walked
 *    from its highest index down;
 *  - each particle of cell m1 scans the 14-cell half stencil; a partner j2
 *    is kept when (m1 != m2 || j2 > j1) and r^2 < (cf+skin)^2.
 * The per-particle lists are returned in the reference's order in a CSR
 * (start[n+1], nb[]).  Because the cell edge is fixed at setup while the skin
 * may grow later (sep_set_skin), pairs with l_cell < r < cf+skin in
 * non-adjacent cells are missed exactly as in the reference.
 * Returns the number of pairs, or -1 when maxpairs is too small.
 */
long ora_pairs_llist(long n, const double *x, const double L[3], const int nsub[3],
		     double cf, double skin, int excl, const int *molindex,
		     const int *bond, const int *angle, const int *dihed,
		     long *start, int *nb, long maxpairs)
{
	static const int ox[14] = {0, 1, 1, 0, -1, 0, 1, 1, 0, -1, -1, -1, 0, 1};
	static const int oy[14] = {0, 0, 1, 1, 1, 0, 0, 1, 1, 1, 0, -1, -1, -1};
	static const int oz[14] = {0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1};
	const long nc2 = (long)nsub[0] * nsub[1], nc3 = nc2 * nsub[2];
	const double rl2 = (cf + skin) * (cf + skin);
	double lsub[3];
	for (int k = 0; k < 3; k++) lsub[k] = L[k] / nsub[k];

	long *head = malloc(sizeof(long) * nc3), *next = malloc(sizeof(long) * n);
	int **tmp = malloc(sizeof(int *) * n);
	long *cnt = calloc(n, sizeof(long)), *cap = malloc(sizeof(long) * n);
	for (long c = 0; c < nc3; c++) head[c] = -1;
	for (long i = 0; i < n; i++) {
		long c = (long)(x[3 * i] / lsub[0]) + (long)(x[3 * i + 1] / lsub[1]) * nsub[0] +
			 (long)(x[3 * i + 2] / lsub[2]) * nc2;
		if (c < 0 || c >= nc3) c = c < 0 ? 0 : nc3 - 1;
		next[i] = head[c];
		head[c] = i;
		cap[i] = 64;
		tmp[i] = malloc(sizeof(int) * cap[i]);
	}
	for (int cz = 0; cz < nsub[2]; cz++)
		for (int cy = 0; cy < nsub[1]; cy++)
			for (int cx = 0; cx < nsub[0]; cx++) {
				long m1 = cz * nc2 + (long)cy * nsub[0] + cx;
				for (long j1 = head[m1]; j1 != -1; j1 = next[j1]) {
					for (int s = 0; s < 14; s++) {
						int mx = cx + ox[s], my = cy + oy[s], mz = cz + oz[s];
						if (mx == nsub[0]) mx = 0; else if (mx == -1) mx = nsub[0] - 1;
						if (my == nsub[1]) my = 0; else if (my == -1) my = nsub[1] - 1;
						if (mz == nsub[2]) mz = 0;
						long m2 = mz * nc2 + (long)my * nsub[0] + mx;
						for (long j2 = head[m2]; j2 != -1; j2 = next[j2]) {
							if (!(m1 != m2 || j2 > j1)) continue;
							if (excl && ora_excluded(excl, j1, j2, molindex, bond, angle, dihed))
								continue;
							double d[3];
							if (ora_sep(x, j1, j2, L, d) < rl2) {
								if (cnt[j1] == cap[j1]) {
									cap[j1] *= 2;
									tmp[j1] = realloc(tmp[j1], sizeof(int) * cap[j1]);
								}
								tmp[j1][cnt[j1]++] = (int)j2;
							}
						}
					}
				}
			}
	long total = 0;
	for (long i = 0; i < n; i++) {
		start[i] = total;
		for (long k = 0; k < cnt[i]; k++) {
			if (total < maxpairs) nb[total] = tmp[i][k];
			total++;
		}
		free(tmp[i]);
	}
	start[n] = total;
	free(tmp); free(cnt); free(cap); free(head); free(next);
	return total <= maxpairs ? total : -1;
}

/*
 * Pair-potential kinds.  ORA_POT_LJ*: the built-in callbacks of
 * source/sepmisc.c:115-165 (unit sigma/epsilon; shift 0, SEP_LJCF2 or 1.0);
 * ORA_POT_LJPARAM: the inlined Lennard-Jones of sep_force_lj with
 * p = {cf, eps, sigma, aw} (source/sepprfrc.c:782-1000), whose force factor
 * is 48 eps (s^6)(s^6 - aw/2) * sigma^2/r^2 with s = sigma/r, and whose shift is
 * 4 eps ((sigma/cf)^12 - aw (sigma/cf)^6).
 */
enum { ORA_POT_LJ = 0, ORA_POT_LJSHIFT = 1, ORA_POT_WCA = 2, ORA_POT_LJPARAM = 3 };
#define ORA_LJCF2 0.016316891136

static inline void ora_pot(int kind, const double *p, double r2, double *ft, double *u)
{
	if (kind == ORA_POT_LJPARAM) {
		const double eps = p[1], sigma = p[2], aw = p[3], cf = p[0];
		const double shift = 4.0 * eps * (pow(sigma / cf, 12.) - aw * pow(sigma / cf, 6.));
		double rri = sigma * sigma / r2, rri3 = rri * rri * rri;
		*ft = 48.0 * eps * rri3 * (rri3 - 0.5 * aw) * rri;
		*u = 4.0 * eps * rri3 * (rri3 - aw) - shift;
		return;
	}
	double rri = 1.0 / r2, rri3 = rri * rri * rri;
	*ft = 48.0 * rri3 * (rri3 - 0.5) * rri;
	*u = 4.0 * rri3 * (rri3 - 1.0);
	if (kind == ORA_POT_LJSHIFT) *u += ORA_LJCF2;
	else if (kind == ORA_POT_WCA) *u += 1.0;
}

static inline int ora_typematch(char ti, char tj, const char *types)
{
	return (ti == types[0] && tj == types[1]) || (ti == types[1] && tj == types[0]);
}

/*
 * Pair forces over a CSR half list (or any unordered pair list): for every
 * listed pair with matching types and r^2 < cf^2 add f = ft r to i and -f to
 * j, sum the energy and the configurational tensor pot_P[k][kk] += f_k r_kk
 * (source/sepprfrc.c:94-224 and :782-923).  `epot` receives the plain sum;
 * whether the caller assigns or adds it is the caller's business.
 */
void ora_pair_forces(long n, const double *x, const char *type, const double L[3],
		     const char *types, int kind, const double *p, double cf,
		     const long *start, const int *nb, double *f, double *epot, double *potP)
{
	const double cf2 = cf * cf;
	double e = 0.0;
	for (long i = 0; i < n; i++) {
		if (type[i] != types[0] && type[i] != types[1]) continue;
		for (long s = start[i]; s < start[i + 1]; s++) {
			long j = nb[s];
			if (!ora_typematch(type[i], type[j], types)) continue;
			double d[3], r2 = ora_sep(x, i, j, L, d), ft, u;
			if (r2 >= cf2) continue;
			ora_pot(kind, p, r2, &ft, &u);
			for (int k = 0; k < 3; k++) {
				double fk = ft * d[k];
				f[3 * i + k] += fk;
				f[3 * j + k] -= fk;
				for (int kk = 0; kk < 3; kk++) potP[3 * k + kk] += fk * d[kk];
			}
			e += u;
		}
	}
	*epot = e;
}

/*
 * Shifted-force Coulomb over a CSR half list (source/sepcoulomb.c:96-160):
 * particles with |z| < DBL_EPSILON are skipped; ft = zi zj (1/r^2 - 1/cf^2)/r,
 * u = zi zj (1/r + (r - cf)/cf^2 - 1/cf).  The serial reference adds the full
 * energy; its OpenMP variant halves it (source/sepcoulomb.c:226-227), which
 * this oracle does not reproduce.
 */
void ora_coulomb_sf(long n, const double *x, const double *z, const double L[3], double cf,
		    const long *start, const int *nb, double *f, double *ecoul, double *potP)
{
	const double cf2 = cf * cf, icf2 = 1.0 / cf2, icf = 1.0 / cf;
	double e = 0.0;
	for (long i = 0; i < n; i++) {
		if (fabs(z[i]) < 2.220446049250313e-16) continue;
		for (long s = start[i]; s < start[i + 1]; s++) {
			long j = nb[s];
			double d[3], r2 = ora_sep(x, i, j, L, d);
			if (r2 >= cf2) continue;
			double zz = z[i] * z[j], r = sqrt(r2);
			double ft = zz * (1.0 / r2 - icf2) / r;
			for (int k = 0; k < 3; k++) {
				double fk = ft * d[k];
				f[3 * i + k] += fk;
				f[3 * j + k] -= fk;
				for (int kk = 0; kk < 3; kk++) potP[3 * k + kk] += fk * d[kk];
			}
			e += zz * (1.0 / r + (r - cf) * icf2 - icf);
		}
	}
	*ecoul = e;
}

/*
 * Nose-Hoover friction (source/sepintgr.c:149-168): ekin = sum m v^2 / (2n),
 * T = 0.666667 ekin, alpha += dt/tau^2 (T/T0 - 1), f -= alpha m v.
 */
void ora_nosehoover(long n, const double *v, const double *m, double *f,
		    double T0, double *alpha, double tau, double dt)
{
	double ek = 0.0;
	for (long i = 0; i < n; i++)
		for (int k = 0; k < 3; k++) ek += v[3 * i + k] * v[3 * i + k] * m[i];
	ek = 0.5 * ek / n;
	double T = 0.666667 * ek;
	*alpha = *alpha + dt / (tau * tau) * (T / T0 - 1.0);
	for (long i = 0; i < n; i++)
		for (int k = 0; k < 3; k++) f[3 * i + k] -= *alpha * m[i] * v[3 * i + k];
}

/*
 * Leap-frog step with periodic wrap and the skin test
 * (source/sepintgr.c:18-40 sep_periodic, :42-88 sep_leapfrog):
 * a = f/m; v += a dt; x += v dt; vt = v - a dt/2 enters ekin and kin_P; a
 * coordinate above L or below 0 is moved by one box length with the crossing
 * counters updated; d^2 = |x + cross_neighb L - xn|^2 feeds max_dist2; when
 * sqrt(max_dist2) > skin/2 the update flag is raised, the counter incremented,
 * xn = x and cross_neighb = 0.  Returns 1 when an update was flagged.
 * ekin receives 0.5 sum m vt^2 (added), kinP accumulates.
 */
int ora_leapfrog(long n, double *x, double *v, const double *f, double *a, const double *m,
		 int *cross_neighb, int *crossings, double *xn, const double L[3],
		 double dt, double skin, double *max_dist2, double *ekin, double *kinP)
{
	double sum = 0.0;
	for (long i = 0; i < n; i++) {
		double vt[3], d2 = 0.0;
		for (int k = 0; k < 3; k++) {
			long q = 3 * i + k;
			a[q] = f[q] / m[i];
			v[q] += a[q] * dt;
			x[q] += v[q] * dt;
			vt[k] = v[q] - 0.5 * a[q] * dt;
			sum += vt[k] * vt[k] * m[i];
		}
		for (int k = 0; k < 3; k++) {
			long q = 3 * i + k;
			if (x[q] > L[k]) { x[q] -= L[k]; cross_neighb[q]++; crossings[q]++; }
			else if (x[q] < 0.0) { x[q] += L[k]; cross_neighb[q]--; crossings[q]--; }
			double r = (x[q] + cross_neighb[q] * L[k]) - xn[q];
			d2 += r * r;
		}
		if (d2 > *max_dist2) *max_dist2 = d2;
		for (int k = 0; k < 3; k++)
			for (int kk = 0; kk < 3; kk++) kinP[3 * k + kk] += vt[k] * vt[kk] * m[i];
	}
	int flag = 0;
	if (sqrt(*max_dist2) > 0.5 * skin) {
		flag = 1;
		memcpy(xn, x, sizeof(double) * 3 * n);
		memset(cross_neighb, 0, sizeof(int) * 3 * n);
	}
	*ekin += 0.5 * sum;
	return flag;
}

/* harmonic bonds of one type (source/sepmol.c:372-415) */
void ora_stretch_harmonic(long nb, const unsigned *blist, int type, double l0, double ks,
			  const double *x, const double L[3], double *f, double *epot,
			  double *potP, double *potPbond)
{
	for (long b = 0; b < nb; b++) {
		if ((int)blist[3 * b + 2] != type) continue;
		long i = blist[3 * b], j = blist[3 * b + 1];
		double d[3], r2 = ora_sep(x, i, j, L, d), r = sqrt(r2);
		double ft = -ks * (r - l0) / r;
		for (int k = 0; k < 3; k++) {
			double fk = ft * d[k];
			f[3 * i + k] += fk;
			f[3 * j + k] -= fk;
			for (int kk = 0; kk < 3; kk++) {
				potP[3 * k + kk] += fk * d[kk];
				potPbond[3 * k + kk] += fk * d[kk];
			}
		}
		*epot += 0.5 * ks * (r - l0) * (r - l0);
	}
}

/* bond vectors r_ab and r_bc with the minimum image (source/sepmol.c:438-444) */
static void ora_two_vectors(const double *x, long a, long b, long c, const double L[3],
			    double d1[3], double d2[3])
{
	for (int k = 0; k < 3; k++) {
		d1[k] = ora_wrap(x[3 * b + k] - x[3 * a + k], L[k]);
		d2[k] = ora_wrap(x[3 * c + k] - x[3 * b + k], L[k]);
	}
}

/*
 * Angles of one type.  cossq != 0: sep_angle_cossq (source/sepmol.c:418-466),
 * prefactor -k (cos - cos(pi - angle0)); otherwise sep_angle_harmonic
 * (:469-517), prefactor -k (theta - angle0) with theta = pi - acos(c12/cD).
 * Both apply the prefactor to the same cosine-gradient vectors, exactly as
 * the reference does (for the harmonic form that is not the gradient of its
 * energy; the difference is a factor 1/sin(theta)).  No virial contribution.
 */
void ora_angles(long na, const unsigned *alist, int type, double angle0, double kang,
		int cossq, const double *x, const double L[3], double *f, double *epot)
{
	const double pi = 3.14159265358979;
	const double c0 = cos(pi - angle0);
	for (long t = 0; t < na; t++) {
		if ((int)alist[4 * t + 3] != type) continue;
		long a = alist[4 * t], b = alist[4 * t + 1], c = alist[4 * t + 2];
		double d1[3], d2[3];
		ora_two_vectors(x, a, b, c, L, d1, d2);
		double c11 = d1[0] * d1[0] + d1[1] * d1[1] + d1[2] * d1[2];
		double c12 = d1[0] * d2[0] + d1[1] * d2[1] + d1[2] * d2[2];
		double c22 = d2[0] * d2[0] + d2[1] * d2[1] + d2[2] * d2[2];
		double cD = sqrt(c11 * c22), cc = c12 / cD, pref;
		if (cossq) {
			pref = -kang * (cc - c0);
			*epot += 0.5 * kang * (cc - c0) * (cc - c0);
		} else {
			double th = pi - acos(cc);
			pref = -kang * (th - angle0);
			*epot += 0.5 * kang * (th - angle0) * (th - angle0);
		}
		for (int k = 0; k < 3; k++) {
			double f1 = pref * ((c12 / c11) * d1[k] - d2[k]) / cD;
			double f2 = pref * (d1[k] - (c12 / c22) * d2[k]) / cD;
			f[3 * a + k] += f1;
			f[3 * b + k] += -f1 - f2;
			f[3 * c + k] += f2;
		}
	}
}

/* Ryckaert-Bellemans torsions of one type in Rapaport's form
 * (source/sepmol.c:520-587); no virial contribution */
void ora_torsion_rb(long nd, const unsigned *dlist, int type, const double g[6],
		    const double *x, const double L[3], double *f, double *epot)
{
	for (long t = 0; t < nd; t++) {
		if ((int)dlist[5 * t + 4] != type) continue;
		long a = dlist[5 * t], b = dlist[5 * t + 1], c = dlist[5 * t + 2], dd = dlist[5 * t + 3];
		double r1[3], r2[3], r3[3];
		for (int k = 0; k < 3; k++) {
			r1[k] = ora_wrap(x[3 * b + k] - x[3 * a + k], L[k]);
			r2[k] = ora_wrap(x[3 * c + k] - x[3 * b + k], L[k]);
			r3[k] = ora_wrap(x[3 * dd + k] - x[3 * c + k], L[k]);
		}
#define ORA_DOT(u, w) ((u)[0] * (w)[0] + (u)[1] * (w)[1] + (u)[2] * (w)[2])
		double c11 = ORA_DOT(r1, r1), c12 = ORA_DOT(r1, r2), c13 = ORA_DOT(r1, r3);
		double c22 = ORA_DOT(r2, r2), c23 = ORA_DOT(r2, r3), c33 = ORA_DOT(r3, r3);
#undef ORA_DOT
		double cA = c13 * c22 - c12 * c23;
		double cB1 = c11 * c22 - c12 * c12, cB2 = c22 * c33 - c23 * c23;
		double cD = sqrt(cB1 * cB2), cc = cA / cD;
		double pref = -(g[1] + (2. * g[2] + (3. * g[3] + (4. * g[4] + 5. * g[5] * cc) * cc) * cc) * cc);
		double t1 = cA, t2 = c11 * c23 - c12 * c13, t3 = -cB1;
		double t4 = cB2, t5 = c13 * c23 - c12 * c33, t6 = -cA;
		double cR1 = c12 / c22, cR2 = c23 / c22;
		for (int k = 0; k < 3; k++) {
			double f1 = pref * c22 * (t1 * r1[k] + t2 * r2[k] + t3 * r3[k]) / (cD * cB1);
			double f2 = pref * c22 * (t4 * r1[k] + t5 * r2[k] + t6 * r3[k]) / (cD * cB2);
			f[3 * a + k] += f1;
			f[3 * b + k] += -(1.0 + cR1) * f1 + cR2 * f2;
			f[3 * c + k] += cR1 * f1 - (1.0 + cR2) * f2;
			f[3 * dd + k] += f2;
		}
		*epot += g[0] + (g[1] + (g[2] + (g[3] + (g[4] + g[5] * cc) * cc) * cc) * cc) * cc;
	}
}

/*
 * Complete plain-LJ loop, used for energy-drift references and as the timed
 * CPU baseline: per step reset, linked-cell half-list rebuild when flagged,
 * pair forces with Newton's third law (OpenMP over i with a per-thread force
 * array, as the reference's threaded path at source/sepprfrc.c:108-150),
 * optional Nose-Hoover, leap-frog.  The rebuild uses the reference's cell
 * grid rule (nsub from cf + 0.25) and 14-cell stencil via ora_pairs_llist.
 * kind/p select the potential as in ora_pair_forces.  etot_trace (optional,
 * nsteps entries) receives (epot + ekin)/n per step; the final epot, ekin,
 * pot_P, kin_P are written to out[0], out[1], out[2..10], out[11..19];
 * out[20] = number of list updates.  nthreads <= 0 uses the OpenMP default.
 * Returns 0, or -1 on allocation failure.
 */
int ora_run_lj(long n, double *x, double *v, const double *m, const char *type,
	       const double L[3], int kind, const double *p, double cf, double skin,
	       double dt, long nsteps, int nh, double T0, double tau, double *alpha,
	       int nthreads, double *etot_trace, double *out)
{
#ifdef _OPENMP
	if (nthreads > 0) omp_set_num_threads(nthreads);
#else
	(void)nthreads;
#endif
	int nsub[3];
	for (int k = 0; k < 3; k++) nsub[k] = ora_nsubbox(cf, 0.25, L[k]);
	double *f = calloc(3 * n, sizeof(double)), *a = calloc(3 * n, sizeof(double));
	double *xn = calloc(3 * n, sizeof(double));
	int *cn = calloc(3 * n, sizeof(int)), *cr = calloc(3 * n, sizeof(int));
	long *start = malloc(sizeof(long) * (n + 1));
	long maxp = n * 200 + 1000;
	int *nb = malloc(sizeof(int) * maxp);
	if (!f || !a || !xn || !cn || !cr || !start || !nb) return -1;
	const char types[2] = {type[0], type[0]};
	int flag = 1;
	unsigned nupd = 0;
	double epot = 0, ekin = 0, potP[9], kinP[9];
	for (long step = 0; step < nsteps; step++) {
		double maxd2 = 0.0;
		memset(f, 0, sizeof(double) * 3 * n);
		memset(potP, 0, sizeof potP);
		memset(kinP, 0, sizeof kinP);
		ekin = 0.0;
		if (flag) {
			long np = ora_pairs_llist(n, x, L, nsub, cf, skin, 0, NULL, NULL, NULL, NULL,
						  start, nb, maxp);
			if (np < 0) {
				maxp = start[n] + 1000;
				nb = realloc(nb, sizeof(int) * maxp);
				ora_pairs_llist(n, x, L, nsub, cf, skin, 0, NULL, NULL, NULL, NULL,
						start, nb, maxp);
			}
			flag = 0;
		}
		/* threaded Newton-3 force loop with a private force array per thread */
		double e = 0.0, pP[9] = {0};
		const double cf2 = cf * cf;
#pragma omp parallel
		{
			double *fl = calloc(3 * n, sizeof(double));
			double el = 0.0, pl[9] = {0};
#pragma omp for schedule(dynamic, 64)
			for (long i = 0; i < n; i++) {
				for (long s = start[i]; s < start[i + 1]; s++) {
					long j = nb[s];
					if (!ora_typematch(type[i], type[j], types)) continue;
					double d[3], r2 = ora_sep(x, i, j, L, d), ft, u;
					if (r2 >= cf2) continue;
					ora_pot(kind, p, r2, &ft, &u);
					for (int k = 0; k < 3; k++) {
						double fk = ft * d[k];
						fl[3 * i + k] += fk;
						fl[3 * j + k] -= fk;
						for (int kk = 0; kk < 3; kk++) pl[3 * k + kk] += fk * d[kk];
					}
					el += u;
				}
			}
#pragma omp critical
			{
				for (long q = 0; q < 3 * n; q++) f[q] += fl[q];
				for (int k = 0; k < 9; k++) pP[k] += pl[k];
				e += el;
			}
			free(fl);
		}
		epot = e;
		memcpy(potP, pP, sizeof pP);
		if (nh) ora_nosehoover(n, v, m, f, T0, alpha, tau, dt);
		if (ora_leapfrog(n, x, v, f, a, m, cn, cr, xn, L, dt, skin, &maxd2, &ekin, kinP)) {
			flag = 1;
			nupd++;
		}
		if (etot_trace) etot_trace[step] = (epot + ekin) / n;
	}
	if (out) {
		out[0] = epot;
		out[1] = ekin;
		for (int k = 0; k < 9; k++) { out[2 + k] = potP[k]; out[11 + k] = kinP[k]; }
		out[20] = nupd;
	}
	free(f); free(a); free(xn); free(cn); free(cr); free(start); free(nb);
	return 0;
}

/* ---- gradients of an MD loss (the adjoint's oracle) -------------------------
 *
 * The loss of the NVE prgs loop with sep_force_lj (param = {cf, eps, sigma,
 * aw}) and sep_leapfrog (source/sepprfrc.c:743-1000, source/sepintgr.c:42-88):
 *     L = (1/K) sum_{n<K} ( epot_n + (tr kin_P_n + tr pot_P_n) / 3V )
 * in FP64, serial, brute-force pairs (small systems only).  ora_lj_adjoint
 * returns its gradient by the reverse sweep over stored states; the FD test
 * pins it against ora_lj_loss. */

/* per-pair functions of s = r^2 for the reference's LJ force scalar phi
 * (F_i += phi d), energy u, virial w = phi s, their s-derivatives, and their
 * eps- and sigma-derivatives */
typedef struct { double phi, u, phis, us, ws, phie, ue, phisg, usg; } ora_pairfn;

static void ora_lj_pairfn(const double *p, double s, ora_pairfn *o)
{
	const double cf = p[0], eps = p[1], sig = p[2], aw = p[3], awh = 0.5 * aw;
	const double sr = sig / cf, sr6 = pow(sr, 6.0);
	const double shift = -4.0 * eps * (sr6 * sr6 - aw * sr6);
	const double dshift_sig = -24.0 * eps / sig * (2.0 * sr6 * sr6 - aw * sr6);
	const double q = sig * sig / s, s6 = q * q * q;
	o->phi = 48.0 * eps * q * s6 * (s6 - awh);
	o->u = 4.0 * eps * s6 * (s6 - aw) + shift;
	o->phis = -48.0 * eps * q * s6 * (7.0 * s6 - 4.0 * awh) / s;
	o->us = -12.0 * eps * s6 * (2.0 * s6 - aw) / s;
	o->ws = -144.0 * eps * q * s6 * (2.0 * s6 - awh);
	o->phie = o->phi / eps;
	o->ue = o->u / eps;
	o->phisg = 96.0 * eps * q * s6 * (7.0 * s6 - 4.0 * awh) / sig;
	o->usg = 24.0 * eps / sig * s6 * (2.0 * s6 - aw) + dshift_sig;
}

/* one force evaluation: F (3n), epot, tr pot_P */
static void ora_lj_forces_brute(long n, const double *x, const double L[3], const double *p,
				double *F, double *epot, double *trw)
{
	const double cf2 = p[0] * p[0];
	memset(F, 0, sizeof(double) * 3 * n);
	double e = 0.0, w = 0.0;
	for (long i = 0; i < n; i++)
		for (long j = i + 1; j < n; j++) {
			double d[3];
			const double s = ora_sep(x, i, j, L, d);
			if (s >= cf2) continue;
			ora_pairfn f;
			ora_lj_pairfn(p, s, &f);
			for (int k = 0; k < 3; k++) {
				F[3 * i + k] += f.phi * d[k];
				F[3 * j + k] -= f.phi * d[k];
			}
			e += f.u;
			w += f.phi * s;
		}
	*epot = e;
	*trw = w;
}

static void ora_wrap_all(double *x, const double L[3], long n)
{
	for (long i = 0; i < n; i++)
		for (int k = 0; k < 3; k++) {
			x[3 * i + k] -= L[k] * floor(x[3 * i + k] / L[k]);
			if (x[3 * i + k] >= L[k]) x[3 * i + k] -= L[k];
		}
}

double ora_lj_loss(long n, const double *x0, const double *v0, const double *m, const double L[3],
		   const double *p, double dt, long nsteps)
{
	double *x = malloc(sizeof(double) * 3 * n), *u = malloc(sizeof(double) * 3 * n);
	double *F = malloc(sizeof(double) * 3 * n);
	if (!x || !u || !F) return NAN;
	memcpy(x, x0, sizeof(double) * 3 * n);
	memcpy(u, v0, sizeof(double) * 3 * n);
	const double V = L[0] * L[1] * L[2];
	double loss = 0.0;
	for (long step = 0; step < nsteps; step++) {
		double ep, trw, trk = 0.0;
		ora_lj_forces_brute(n, x, L, p, F, &ep, &trw);
		for (long i = 0; i < n; i++)
			for (int k = 0; k < 3; k++) {
				const double a = F[3 * i + k] / m[i];
				u[3 * i + k] += a * dt;
				x[3 * i + k] += u[3 * i + k] * dt;
				const double vt = u[3 * i + k] - 0.5 * a * dt;
				trk += m[i] * vt * vt;
			}
		ora_wrap_all(x, L, n);
		loss += ep + (trk + trw) / (3.0 * V);
	}
	free(x); free(u); free(F);
	return loss / nsteps;
}

int ora_lj_adjoint(long n, const double *x0, const double *v0, const double *m, const double L[3],
		   const double *p, double dt, long nsteps, double *dL_deps, double *dL_dsig,
		   double *dL_dx0)
{
	const long K = nsteps;
	double *X = malloc(sizeof(double) * 3 * n * (K + 1)), *U = malloc(sizeof(double) * 3 * n * (K + 1));
	double *F = malloc(sizeof(double) * 3 * n), *lx = calloc(3 * n, sizeof(double));
	double *lu = calloc(3 * n, sizeof(double)), *h = malloc(sizeof(double) * 3 * n);
	if (!X || !U || !F || !lx || !lu || !h) return -1;
	memcpy(X, x0, sizeof(double) * 3 * n);
	memcpy(U, v0, sizeof(double) * 3 * n);
	for (long s = 0; s < K; s++) {
		double *x = X + 3 * n * s, *u = U + 3 * n * s, *x1 = X + 3 * n * (s + 1), *u1 = U + 3 * n * (s + 1);
		double ep, trw;
		ora_lj_forces_brute(n, x, L, p, F, &ep, &trw);
		for (long q = 0; q < 3 * n; q++) {
			u1[q] = u[q] + F[q] / m[q / 3] * dt;
			x1[q] = x[q] + u1[q] * dt;
		}
		ora_wrap_all(x1, L, n);
	}
	const double V = L[0] * L[1] * L[2], cK = 1.0 / K, cf2 = p[0] * p[0];
	double ge = 0.0, gs = 0.0;
	for (long s = K - 1; s >= 0; s--) {
		const double *x = X + 3 * n * s, *u = U + 3 * n * s, *u1 = U + 3 * n * (s + 1);
		for (long q = 0; q < 3 * n; q++) {
			const double mi = m[q / 3];
			const double kin = cK * mi * 0.5 * (u[q] + u1[q]) / (3.0 * V);
			const double g = lu[q] + dt * lx[q] + kin;
			lu[q] = g + kin;
			h[q] = dt / mi * g;
		}
		for (long i = 0; i < n; i++)
			for (long j = i + 1; j < n; j++) {
				double d[3];
				const double sq = ora_sep(x, i, j, L, d);
				if (sq >= cf2) continue;
				ora_pairfn f;
				ora_lj_pairfn(p, sq, &f);
				double dh[3], ddh = 0.0, dhi = 0.0, dhj = 0.0;
				for (int k = 0; k < 3; k++) {
					dh[k] = h[3 * i + k] - h[3 * j + k];
					ddh += d[k] * dh[k];
					dhi += d[k] * h[3 * i + k];
					dhj += d[k] * h[3 * j + k];
				}
				const double c2 = 2.0 * f.phis * ddh + 2.0 * cK * (f.us + f.ws / (3.0 * V));
				for (int k = 0; k < 3; k++) {
					const double t = f.phi * dh[k] + c2 * d[k];
					lx[3 * i + k] += t;
					lx[3 * j + k] -= t;
				}
				ge += f.phie * (dhi - dhj) + cK * (f.ue + f.phie * sq / (3.0 * V));
				gs += f.phisg * (dhi - dhj) + cK * (f.usg + f.phisg * sq / (3.0 * V));
			}
	}
	*dL_deps = ge;
	*dL_dsig = gs;
	memcpy(dL_dx0, lx, sizeof(double) * 3 * n);
	free(X); free(U); free(F); free(lx); free(lu); free(h);
	return 0;
}

/* ---- typed loss and adjoint: one LJ parameter set per type pair ------------
 *
 * The NVE prgs loop with one sep_force_lj call per unordered type pair {a, b}
 * (param_ab = {cf, eps, sigma, aw}; source/sepprfrc.c:743-1000: the term of
 * types "ab" applies to every pair whose types are a and b in either order,
 * and the energies of the calls add) and sep_leapfrog
 * (source/sepintgr.c:42-88).  P holds nt x nt parameter sets of 4 doubles,
 * symmetric (P[a][b] == P[b][a]); eps = 0 switches a pair type off.  Pairs
 * are found each step through a linked-cell list of cells at least the
 * largest cut-off wide (every pair once, i < j), or by brute force when a
 * box side holds fewer than three such cells. */

typedef struct { long np, cap; int *ij; } ora_plist;

static int ora_plist_push(ora_plist *pl, long i, long j)
{
	if (pl->np == pl->cap) {
		long nc = pl->cap ? 2 * pl->cap : 4096;
		int *q = realloc(pl->ij, sizeof(int) * 2 * nc);
		if (!q) return -1;
		pl->ij = q;
		pl->cap = nc;
	}
	pl->ij[2 * pl->np] = (int)i;
	pl->ij[2 * pl->np + 1] = (int)j;
	pl->np++;
	return 0;
}

/* every unordered pair i < j with r^2 < rmax^2 (minimum image) */
static int ora_halfpairs(long n, const double *x, const double L[3], double rmax, ora_plist *pl)
{
	const double r2max = rmax * rmax;
	int nc[3];
	double d[3];
	pl->np = 0;
	for (int k = 0; k < 3; k++) nc[k] = (int)floor(L[k] / rmax);
	if (nc[0] < 3 || nc[1] < 3 || nc[2] < 3) {
		for (long i = 0; i < n; i++)
			for (long j = i + 1; j < n; j++)
				if (ora_sep(x, i, j, L, d) < r2max && ora_plist_push(pl, i, j)) return -1;
		return 0;
	}
	const long ncell = (long)nc[0] * nc[1] * nc[2];
	long *head = malloc(sizeof(long) * ncell), *next = malloc(sizeof(long) * n);
	if (!head || !next) { free(head); free(next); return -1; }
	for (long c = 0; c < ncell; c++) head[c] = -1;
	int (*cell)[3] = malloc(sizeof(int) * 3 * n);
	if (!cell) { free(head); free(next); return -1; }
	for (long i = 0; i < n; i++) {
		for (int k = 0; k < 3; k++) {
			int c = (int)floor(x[3 * i + k] / L[k] * nc[k]);
			c = c < 0 ? 0 : (c >= nc[k] ? nc[k] - 1 : c);
			cell[i][k] = c;
		}
		const long c = cell[i][0] + (long)nc[0] * (cell[i][1] + (long)nc[1] * cell[i][2]);
		next[i] = head[c];
		head[c] = i;
	}
	int rc = 0;
	for (long i = 0; i < n && !rc; i++)
		for (int oz = -1; oz <= 1; oz++)
			for (int oy = -1; oy <= 1; oy++)
				for (int ox = -1; ox <= 1; ox++) {
					const int cx = (cell[i][0] + ox + nc[0]) % nc[0];
					const int cy = (cell[i][1] + oy + nc[1]) % nc[1];
					const int cz = (cell[i][2] + oz + nc[2]) % nc[2];
					for (long j = head[cx + (long)nc[0] * (cy + (long)nc[1] * cz)]; j != -1; j = next[j])
						if (j > i && ora_sep(x, i, j, L, d) < r2max && ora_plist_push(pl, i, j))
							rc = -1;
				}
	free(head); free(next); free(cell);
	return rc;
}

static double ora_maxcf(int nt, const double *P)
{
	double c = 0.0;
	for (int k = 0; k < nt * nt; k++)
		if (P[4 * k + 1] != 0.0 && P[4 * k] > c) c = P[4 * k];
	return c;
}

/* forces, energy and tr pot_P of the typed terms over the pairs of pl */
static void ora_ljt_forces(long n, const double *x, const int *type, const double L[3], int nt,
			   const double *P, const ora_plist *pl, double *F, double *epot, double *trw)
{
	memset(F, 0, sizeof(double) * 3 * n);
	double e = 0.0, w = 0.0, d[3];
	for (long k = 0; k < pl->np; k++) {
		const long i = pl->ij[2 * k], j = pl->ij[2 * k + 1];
		const double *p = P + 4 * (type[i] * nt + type[j]);
		if (p[1] == 0.0) continue;
		const double s = ora_sep(x, i, j, L, d);
		if (s >= p[0] * p[0]) continue;
		ora_pairfn f;
		ora_lj_pairfn(p, s, &f);
		for (int q = 0; q < 3; q++) {
			F[3 * i + q] += f.phi * d[q];
			F[3 * j + q] -= f.phi * d[q];
		}
		e += f.u;
		w += f.phi * s;
	}
	*epot = e;
	*trw = w;
}

double ora_ljt_loss(long n, const double *x0, const double *v0, const double *m, const int *type,
		    const double L[3], int nt, const double *P, double dt, long nsteps)
{
	double *x = malloc(sizeof(double) * 3 * n), *u = malloc(sizeof(double) * 3 * n);
	double *F = malloc(sizeof(double) * 3 * n);
	ora_plist pl = {0, 0, NULL};
	if (!x || !u || !F) { free(x); free(u); free(F); return NAN; }
	memcpy(x, x0, sizeof(double) * 3 * n);
	memcpy(u, v0, sizeof(double) * 3 * n);
	const double V = L[0] * L[1] * L[2], rmax = ora_maxcf(nt, P);
	double loss = 0.0;
	for (long step = 0; step < nsteps; step++) {
		double ep, trw, trk = 0.0;
		if (ora_halfpairs(n, x, L, rmax, &pl)) { loss = NAN; break; }
		ora_ljt_forces(n, x, type, L, nt, P, &pl, F, &ep, &trw);
		for (long i = 0; i < n; i++)
			for (int k = 0; k < 3; k++) {
				const double a = F[3 * i + k] / m[i];
				u[3 * i + k] += a * dt;
				x[3 * i + k] += u[3 * i + k] * dt;
				const double vt = u[3 * i + k] - 0.5 * a * dt;
				trk += m[i] * vt * vt;
			}
		ora_wrap_all(x, L, n);
		loss += ep + (trk + trw) / (3.0 * V);
	}
	free(x); free(u); free(F); free(pl.ij);
	return loss / nsteps;
}

/* gradient of ora_ljt_loss: dL_deps[a * nt + b] and dL_dsig[a * nt + b]
 * (both orders filled with the gradient of the one shared parameter) and
 * dL_dx0 (3n) */
int ora_ljt_adjoint(long n, const double *x0, const double *v0, const double *m, const int *type,
		    const double L[3], int nt, const double *P, double dt, long nsteps, double *dL_deps,
		    double *dL_dsig, double *dL_dx0)
{
	const long K = nsteps;
	double *X = malloc(sizeof(double) * 3 * n * (K + 1)), *U = malloc(sizeof(double) * 3 * n * (K + 1));
	double *F = malloc(sizeof(double) * 3 * n), *lx = calloc(3 * n, sizeof(double));
	double *lu = calloc(3 * n, sizeof(double)), *h = malloc(sizeof(double) * 3 * n);
	double *ge = calloc(nt * nt, sizeof(double)), *gs = calloc(nt * nt, sizeof(double));
	ora_plist pl = {0, 0, NULL};
	int rc = -1;
	if (!X || !U || !F || !lx || !lu || !h || !ge || !gs) goto out;
	memcpy(X, x0, sizeof(double) * 3 * n);
	memcpy(U, v0, sizeof(double) * 3 * n);
	const double V = L[0] * L[1] * L[2], cK = 1.0 / K, rmax = ora_maxcf(nt, P);
	for (long s = 0; s < K; s++) {
		double *x = X + 3 * n * s, *u = U + 3 * n * s, *x1 = X + 3 * n * (s + 1), *u1 = U + 3 * n * (s + 1);
		double ep, trw;
		if (ora_halfpairs(n, x, L, rmax, &pl)) goto out;
		ora_ljt_forces(n, x, type, L, nt, P, &pl, F, &ep, &trw);
		for (long q = 0; q < 3 * n; q++) {
			u1[q] = u[q] + F[q] / m[q / 3] * dt;
			x1[q] = x[q] + u1[q] * dt;
		}
		ora_wrap_all(x1, L, n);
	}
	for (long s = K - 1; s >= 0; s--) {
		const double *x = X + 3 * n * s, *u = U + 3 * n * s, *u1 = U + 3 * n * (s + 1);
		for (long q = 0; q < 3 * n; q++) {
			const double mi = m[q / 3];
			const double kin = cK * mi * 0.5 * (u[q] + u1[q]) / (3.0 * V);
			const double g = lu[q] + dt * lx[q] + kin;
			lu[q] = g + kin;
			h[q] = dt / mi * g;
		}
		if (ora_halfpairs(n, x, L, rmax, &pl)) goto out;
		for (long k = 0; k < pl.np; k++) {
			const long i = pl.ij[2 * k], j = pl.ij[2 * k + 1];
			const int tp = type[i] * nt + type[j];
			const double *p = P + 4 * tp;
			if (p[1] == 0.0) continue;
			double d[3];
			const double sq = ora_sep(x, i, j, L, d);
			if (sq >= p[0] * p[0]) continue;
			ora_pairfn f;
			ora_lj_pairfn(p, sq, &f);
			double dh[3], ddh = 0.0, dhi = 0.0, dhj = 0.0;
			for (int q = 0; q < 3; q++) {
				dh[q] = h[3 * i + q] - h[3 * j + q];
				ddh += d[q] * dh[q];
				dhi += d[q] * h[3 * i + q];
				dhj += d[q] * h[3 * j + q];
			}
			const double c2 = 2.0 * f.phis * ddh + 2.0 * cK * (f.us + f.ws / (3.0 * V));
			for (int q = 0; q < 3; q++) {
				const double t = f.phi * dh[q] + c2 * d[q];
				lx[3 * i + q] += t;
				lx[3 * j + q] -= t;
			}
			const int tu = type[i] < type[j] ? type[i] * nt + type[j] : type[j] * nt + type[i];
			ge[tu] += f.phie * (dhi - dhj) + cK * (f.ue + f.phie * sq / (3.0 * V));
			gs[tu] += f.phisg * (dhi - dhj) + cK * (f.usg + f.phisg * sq / (3.0 * V));
		}
	}
	for (int a = 0; a < nt; a++)
		for (int b = 0; b < nt; b++) {
			const int tu = a < b ? a * nt + b : b * nt + a;
			dL_deps[a * nt + b] = ge[tu];
			dL_dsig[a * nt + b] = gs[tu];
		}
	memcpy(dL_dx0, lx, sizeof(double) * 3 * n);
	rc = 0;
out:
	free(X); free(U); free(F); free(lx); free(lu); free(h); free(ge); free(gs); free(pl.ij);
	return rc;
}

/* ======================================================================
 * Stochastic dynamics: DPD pair force, Groot-Warren integrator,
 * Fokker-Planck and Langevin (GJF) integrators.
 *
 * The reference draws its random numbers from the C library's rand() in
 * the order its loops visit pairs and particles.  The restatements below
 * take the random numbers as inputs, so they can be driven either by that
 * stream (to pin them against the reference) or by the GPU library's
 * counter-based streams (ora_dpd_uniform, ora_gauss3) to check the GPU.
 * ====================================================================== */

#include <stdint.h>

/* Philox4x32-10 (J. K. Salmon, M. A. Moraes, R. O. Dror, D. E. Shaw,
 * "Parallel random numbers: as easy as 1, 2, 3", SC'11): ten rounds of two
 * 32x32->64 multiplications with the Weyl key schedule. */
void ora_philox(uint32_t c[4], uint32_t k0, uint32_t k1)
{
	for (int r = 0; r < 10; r++) {
		if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
		const uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
		const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
		c[1] = (uint32_t)p1;
		c[3] = (uint32_t)p0;
		c[0] = n0;
		c[2] = n2;
	}
}

/* stream ids of the GPU library's counters (fourth counter word) */
enum { ORA_STREAM_DPD = 1, ORA_STREAM_FP = 2, ORA_STREAM_GJF = 3 };

/* DPD pair uniform in [0, 1) of the GPU library: counter (min gid, max gid,
 * call, DPD), key = seed; 24 bits of the first output word */
double ora_dpd_uniform(uint64_t seed, int gi, int gj, uint32_t call)
{
	uint32_t c[4] = {(uint32_t)(gi < gj ? gi : gj), (uint32_t)(gi < gj ? gj : gi), call, ORA_STREAM_DPD};
	ora_philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
	return (double)(c[0] >> 8) * (1.0 / 16777216.0);
}

/* three standard normal numbers of particle gid for one call of a stream:
 * counter (gid, 0, call, stream); Box-Muller on the output pairs
 * (w0, w1) and (w2, w3), u1 in (0, 1], u2 in [0, 1) */
void ora_gauss3(uint64_t seed, int gid, uint32_t call, int stream, double g[3])
{
	uint32_t c[4] = {(uint32_t)gid, 0u, call, (uint32_t)stream};
	ora_philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
	const double two_pi = 6.283185307179586;
	for (int h = 0; h < 2; h++) {
		const double u1 = (double)((c[2 * h] >> 8) + 1u) * (1.0 / 16777216.0);
		const double u2 = (double)(c[2 * h + 1] >> 8) * (1.0 / 16777216.0);
		const double r = sqrt(-2.0 * log(u1));
		g[2 * h] = r * cos(two_pi * u2);
		if (h == 0) g[1] = r * sin(two_pi * u2);
	}
}

/*
 * DPD pair force of Groot and Warren (source/sepprfrc.c:1007-1104).  Pairs are
 * visited in the order given (i, j) = pairs[2p], pairs[2p+1]; a pair is used
 * when the first particle's type is one of types[0..1], the two types match
 * the pair in either order, and r^2 < cf^2.  With w = 1 - r, rhat = r/|r|,
 * vij = pv_i - pv_j (predicted velocities), gamma = sigma^2 / (2 T):
 *   fC = aij w rhat, fD = -gamma w^2 (rhat . vij) rhat,
 *   fR = sigma w rhat dt^(-1/2) (u - 0.5) 2 sqrt(3),
 * added to i and subtracted from j; epot = sum aij w^2 / 2 (assigned).
 * u: per_pair = 0 consumes uni[] in order, one per used pair (the
 * reference's rand() stream); per_pair = 1 takes uni[p] of the pair's index.
 * The sums go to a separate array that is added to f at the end, as the
 * reference's list form does.  vir (27 doubles, may be NULL) accumulates the
 * virials of the O(N^2) form (source/sepprfrc.c:1196-1206): fC_k r_kk,
 * fR_k r_kk, fD_k r_kk, row-major 3x3 each.
 */
void ora_dpd_forces(long n, const double *x, const double *pv, const char *type, const double L[3],
		    const char *types, double cf, double aij, double temp, double sigma, double dt,
		    long npairs, const int *pairs, const double *uni, int per_pair, double *f, double *epot,
		    double *vir)
{
	const double cf2 = cf * cf, isqrtdt = 1.0 / sqrt(dt), facchk = 2.0 * sqrt(3.0);
	const double gamma = sigma * sigma / (2.0 * temp);
	double *fa = calloc(3 * (size_t)n, sizeof(double));
	double e = 0.0;
	long used = 0;
	for (long p = 0; p < npairs; p++) {
		const int i1 = pairs[2 * p], i2 = pairs[2 * p + 1];
		if (type[i1] != types[0] && type[i1] != types[1]) continue;
		if (!((type[i1] == types[0] && type[i2] == types[1]) || (type[i1] == types[1] && type[i2] == types[0])))
			continue;
		double r[3], r2 = 0.0;
		for (int k = 0; k < 3; k++) {
			r[k] = ora_wrap(x[3 * i1 + k] - x[3 * i2 + k], L[k]);
			r2 += r[k] * r[k];
		}
		if (!(r2 < cf2)) continue;
		const double dij = sqrt(r2), w = 1.0 - dij;
		double rhat[3], dotrv = 0.0;
		for (int k = 0; k < 3; k++) {
			rhat[k] = r[k] / dij;
			dotrv += rhat[k] * (pv[3 * i1 + k] - pv[3 * i2 + k]);
		}
		const double u = per_pair ? uni[p] : uni[used];
		used++;
		const double rn = (u - 0.5) * facchk;
		for (int k = 0; k < 3; k++) {
			const double fC = aij * w * rhat[k];
			const double fD = -gamma * w * w * dotrv * rhat[k];
			const double fR = sigma * w * rhat[k] * isqrtdt * rn;
			fa[3 * i1 + k] += fC + fD + fR;
			fa[3 * i2 + k] -= fC + fD + fR;
			if (vir)
				for (int kk = 0; kk < 3; kk++) {
					vir[3 * k + kk] += fC * r[kk];
					vir[9 + 3 * k + kk] += fR * r[kk];
					vir[18 + 3 * k + kk] += fD * r[kk];
				}
		}
		e += 0.5 * aij * w * w;
	}
	for (long q = 0; q < 3 * n; q++) f[q] += fa[q];
	free(fa);
	*epot = e;
}

/* reference sep_periodic (source/sepintgr.c:17-37): wrap one coordinate
 * set, count crossings, return |x + cross_neighb L - xn|^2 */
static double ora_periodic(long i, double *x, int *cross_neighb, int *crossings, const double *xn,
			   const double L[3])
{
	double d2 = 0.0;
	for (int k = 0; k < 3; k++) {
		const long q = 3 * i + k;
		if (x[q] > L[k]) { x[q] -= L[k]; cross_neighb[q]++; crossings[q]++; }
		else if (x[q] < 0.0) { x[q] += L[k]; cross_neighb[q]--; crossings[q]--; }
		const double ri = (x[q] + cross_neighb[q] * L[k]) - xn[q];
		d2 += ri * ri;
	}
	return d2;
}

/* the skin test shared by the integrators: xn = x, cross_neighb = 0 */
static int ora_skin(long n, const double *x, int *cross_neighb, double *xn, double skin, double max_dist2)
{
	if (!(sqrt(max_dist2) > 0.5 * skin)) return 0;
	memcpy(xn, x, sizeof(double) * 3 * n);
	memset(cross_neighb, 0, sizeof(int) * 3 * n);
	return 1;
}

/*
 * Groot-Warren velocity Verlet (source/sepintgr.c:296-345): a = f/m;
 * v += dt (a + pa)/2 unless stepnow == 0; x += v dt + a dt^2/2;
 * pv = v + lambda dt a; pa = a; ekin += sum m v^2 / 2 and kin_P += m v v^T
 * with the updated v.  Returns 1 when the skin test fired (the reference
 * raises neighb_flag there but does not count the update).
 */
int ora_verlet_dpd(long n, double *x, double *v, const double *f, double *a, const double *m,
		   double *pv, double *pa, double lambda, int stepnow, int *cross_neighb, int *crossings,
		   double *xn, const double L[3], double dt, double skin, double *max_dist2,
		   double *ekin, double *kinP)
{
	double sum = 0.0;
	for (long i = 0; i < n; i++) {
		for (int k = 0; k < 3; k++) {
			const long q = 3 * i + k;
			a[q] = f[q] / m[i];
			if (stepnow > 0) v[q] += 0.5 * dt * (a[q] + pa[q]);
			x[q] += v[q] * dt + 0.5 * dt * dt * a[q];
			pv[q] = v[q] + lambda * dt * a[q];
			pa[q] = a[q];
			sum += v[q] * v[q] * m[i];
		}
		const double d2 = ora_periodic(i, x, cross_neighb, crossings, xn, L);
		if (d2 > *max_dist2) *max_dist2 = d2;
		for (int k = 0; k < 3; k++)
			for (int kk = 0; kk < 3; kk++) kinP[3 * k + kk] += v[3 * i + k] * v[3 * i + kk] * m[i];
	}
	*ekin += 0.5 * sum;
	return ora_skin(n, x, cross_neighb, xn, skin, *max_dist2);
}

/*
 * Fokker-Planck (Brownian) integrator (source/sepintgr.c:235-293): per
 * coordinate a = g sqrt(1/12) sqrt(24 T fric/dt) with g standard normal
 * (gauss[3 i + k]) and fric = T / ldiff; x += dt v (old v);
 * v += dt/m (f - fric v + a); wrap; ekin, kin_P from the new v.  Returns 1
 * when the skin test fired (the reference counts that update).
 */
int ora_fp(long n, double *x, double *v, const double *f, const double *m, const double *ldiff,
	   const double *gauss, double temp, int *cross_neighb, int *crossings, double *xn,
	   const double L[3], double dt, double skin, double *max_dist2, double *ekin, double *kinP)
{
	const double fac = sqrt(1.0 / 12.0);
	double sum = 0.0;
	for (long i = 0; i < n; i++) {
		const double im = 1.0 / m[i], fric = temp / ldiff[i];
		const double gaussfac = sqrt(24 * temp * fric / dt);
		double d2 = 0.0;
		for (int k = 0; k < 3; k++) {
			const long q = 3 * i + k;
			const double ak = gauss[q] * fac * gaussfac;
			x[q] += dt * v[q];
			v[q] += im * dt * (f[q] - fric * v[q] + ak);
			if (x[q] > L[k]) { x[q] -= L[k]; cross_neighb[q]++; crossings[q]++; }
			else if (x[q] < 0.0) { x[q] += L[k]; cross_neighb[q]--; crossings[q]--; }
			sum += v[q] * v[q] * m[i];
			const double ri = (x[q] + cross_neighb[q] * L[k]) - xn[q];
			d2 += ri * ri;
		}
		if (d2 > *max_dist2) *max_dist2 = d2;
		for (int k = 0; k < 3; k++)
			for (int kk = 0; kk < 3; kk++) kinP[3 * k + kk] += v[3 * i + k] * v[3 * i + kk] * m[i];
	}
	*ekin += 0.5 * sum;
	return ora_skin(n, x, cross_neighb, xn, skin, *max_dist2);
}

/*
 * Langevin integrator of Gronbech-Jensen and Farago
 * (source/sepintgr.c:91-146): cc = exp(-alpha dt), fac = sqrt(T (1 - cc^2)),
 * c = alpha dt / (2 m), a' = (1 - c)/(1 + c), b = 1/(1 + c);
 * v = a' v + dt/(2m) (a' prevf + f) + b randn / m; prevf = f;
 * randn = fac g (new draw, gauss[3 i + k]);
 * x += b dt v + b dt^2/(2m) f + b dt/(2m) randn; wrap; ekin and kin_P from
 * the new v.  Returns 1 when the skin test fired (counted).
 */
int ora_langevin_gjf(long n, double *x, double *v, const double *f, double *a, const double *m,
		     double *prevf, double *randn, const double *gauss, double temp, double alpha,
		     int *cross_neighb, int *crossings, double *xn, const double L[3], double dt,
		     double skin, double *max_dist2, double *ekin, double *kinP)
{
	const double cc = exp(-alpha * dt);
	double sum = 0.0;
	for (long i = 0; i < n; i++) {
		const double mass = m[i], imass = 1.0 / mass, imass2 = 0.5 * imass;
		const double fac = sqrt(temp * (1.0 - cc * cc));
		const double c = alpha * dt * imass2, ap = (1.0 - c) / (1.0 + c), b = 1.0 / (1.0 + c);
		for (int k = 0; k < 3; k++) {
			const long q = 3 * i + k;
			v[q] = ap * v[q] + dt * imass2 * (ap * prevf[q] + f[q]) + b * imass * randn[q];
			a[q] = f[q] * imass;
			prevf[q] = f[q];
			sum += v[q] * v[q] * mass;
			randn[q] = fac * gauss[q];
			x[q] += b * dt * v[q] + b * dt * dt * imass2 * f[q] + b * dt * imass2 * randn[q];
		}
		const double d2 = ora_periodic(i, x, cross_neighb, crossings, xn, L);
		if (d2 > *max_dist2) *max_dist2 = d2;
		for (int k = 0; k < 3; k++)
			for (int kk = 0; kk < 3; kk++) kinP[3 * k + kk] += v[3 * i + k] * v[3 * i + kk] * mass;
	}
	*ekin += 0.5 * sum;
	return ora_skin(n, x, cross_neighb, xn, skin, *max_dist2);
}

/* ======================================================================
 * Box changes: compression and the Berendsen barostat
 * (source/sepmisc.c:892-1084).  L, volume and the reference's sub-box grid
 * (nsub, lsub) change with the box; positions are scaled in place and are
 * not wrapped (the next integrator step does that).  update = the system's
 * neighb_update (0: SEP_BRUTE keeps the grid).
 * ====================================================================== */

static void ora_subbox(int k, double cf, double delta, const double L[3], int update, int nsub[3],
		       double lsub[3])
{
	if (update == 0) return;
	nsub[k] = ora_nsubbox(cf, delta, L[k]);
	lsub[k] = L[k] / nsub[k];
}

/* sep_compress_box (:989-1024): returns 0 when the density is within 1e-6
 * of rhoD (nothing changes) */
int ora_compress_box(long n, double *x, double L[3], double *volume, int nsub[3], double lsub[3],
		     double cf, double skin, int update, double rhoD, double xi)
{
	const double density = n / *volume;
	if (fabs(density - rhoD) < 1e-6) return 0;
	if (density > rhoD) xi = 1.0 / xi;
	for (int k = 0; k < 3; k++) L[k] *= xi;
	for (long i = 0; i < 3 * n; i++) x[i] *= xi;
	for (int k = 0; k < 3; k++) ora_subbox(k, cf, skin, L, update, nsub, lsub);
	*volume = L[0] * L[1] * L[2];
	return 1;
}

/* sep_compress_box_dir (:1029-1054) and sep_compress_box_dir_length
 * (:1057-1082): one axis, positions scaled by xi^(1/3) */
static void ora_compress_axis(long n, double *x, double L[3], double *volume, int nsub[3],
			      double lsub[3], double cf, int update, double xi, int dir)
{
	L[dir] *= xi;
	const double scale = pow(xi, 1.0 / 3.0);
	for (long i = 0; i < n; i++) x[3 * i + dir] *= scale;
	ora_subbox(dir, cf, 0.0, L, update, nsub, lsub);
	*volume = L[0] * L[1] * L[2];
}

int ora_compress_box_dir(long n, double *x, double L[3], double *volume, int nsub[3], double lsub[3],
			 double cf, int update, double rhoD, double xi, int dir)
{
	if (!(n / *volume < rhoD)) return 0;
	ora_compress_axis(n, x, L, volume, nsub, lsub, cf, update, xi, dir);
	return 1;
}

int ora_compress_box_dir_length(long n, double *x, double L[3], double *volume, int nsub[3],
				double lsub[3], double cf, int update, double length, double xi, int dir)
{
	if (!(L[dir] > length)) return 0;
	ora_compress_axis(n, x, L, volume, nsub, lsub, cf, update, xi, dir);
	return 1;
}

/* sep_berendsen (:892-916) and sep_berendsen_iso (:920-946):
 * xi = 1 - beta dt (Pd - p); iso = 0 scales L_z by xi, iso = 1 all three
 * edges; positions are scaled by xi^(1/3) on the same axes */
void ora_berendsen(long n, double *x, double L[3], double *volume, int nsub[3], double lsub[3],
		   double cf, int update, double p, double Pd, double beta, double dt, int iso)
{
	const double xi = 1 - beta * dt * (Pd - p);
	const int k0 = iso ? 0 : 2;
	for (int k = k0; k < 3; k++) L[k] *= xi;
	const double scale = pow(xi, 1.0 / 3.0);
	for (long i = 0; i < n; i++)
		for (int k = k0; k < 3; k++) x[3 * i + k] *= scale;
	*volume = L[0] * L[1] * L[2];
	for (int k = k0; k < 3; k++) ora_subbox(k, cf, 0.0, L, update, nsub, lsub);
}

/* ======================================================================
 * Molecular pressure tensor (source/sepmol.c:683-748 centres of mass,
 * :913-959 sep_eval_mol_pressure_tensor; source/sepret.c:85-102).
 * The reference accumulates the intermolecular force matrix F[i][j] (the
 * force molecule j exerts on molecule i) during the pair-force calls and
 * forms the tensor later from the centres of mass at that later time.
 * F is dense nmol x nmol x 3 here (test sizes only).
 * ====================================================================== */

/* F[mi][mj] += f, F[mj][mi] -= f for each pair force f on i from j with both
 * molecule indices set (source/sepprfrc.c:199-204 and :905-910) */
static void ora_fij_add(double *F, int nmol, int mi, int mj, const double f[3])
{
	if (mi < 0 || mj < 0) return;
	for (int k = 0; k < 3; k++) {
		F[((long)mi * nmol + mj) * 3 + k] += f[k];
		F[((long)mj * nmol + mi) * 3 + k] -= f[k];
	}
}

void ora_pair_fij(long n, const double *x, const char *type, const double L[3], const char *types,
		  int kind, const double *p, double cf, const long *start, const int *nb,
		  const int *molindex, int nmol, double *F)
{
	const double cf2 = cf * cf;
	for (long i = 0; i < n; i++) {
		if (type[i] != types[0] && type[i] != types[1]) continue;
		for (long s = start[i]; s < start[i + 1]; s++) {
			const long j = nb[s];
			if (!ora_typematch(type[i], type[j], types)) continue;
			double d[3], r2 = ora_sep(x, i, j, L, d), ft, u;
			if (r2 >= cf2) continue;
			ora_pot(kind, p, r2, &ft, &u);
			const double f[3] = {ft * d[0], ft * d[1], ft * d[2]};
			ora_fij_add(F, nmol, molindex[i], molindex[j], f);
		}
	}
}

/* the shifted-force Coulomb contribution (source/sepcoulomb.c:140-145) */
void ora_coulomb_fij(long n, const double *x, const double *z, const double L[3], double cf,
		     const long *start, const int *nb, const int *molindex, int nmol, double *F)
{
	const double cf2 = cf * cf, icf2 = 1.0 / cf2;
	for (long i = 0; i < n; i++) {
		if (fabs(z[i]) < 2.220446049250313e-16) continue;
		for (long s = start[i]; s < start[i + 1]; s++) {
			const long j = nb[s];
			double d[3], r2 = ora_sep(x, i, j, L, d);
			if (r2 >= cf2) continue;
			const double r = sqrt(r2), ft = z[i] * z[j] * (1.0 / r2 - icf2) / r;
			const double f[3] = {ft * d[0], ft * d[1], ft * d[2]};
			ora_fij_add(F, nmol, molindex[i], molindex[j], f);
		}
	}
}

/* centre of mass (source/sepmol.c:683-729): the chain of atoms first,
 * first+1, ... first+nuau-1 unwrapped bond by bond from the first atom,
 * mass-weighted (masses of those atoms, divided by the molecule mass),
 * wrapped into the box; centre-of-mass velocity (:731-748) over the
 * molecule's atom list (CSR start/atoms) */
void ora_mol_cm(int nmol, const int *first, const int *nuau, const double *mmol, const double *x,
		const double *m, const double L[3], double *cm)
{
	for (int i = 0; i < nmol; i++) {
		const int a0 = first[i];
		double prev[3] = {x[3 * a0], x[3 * a0 + 1], x[3 * a0 + 2]}, c[3] = {0.0, 0.0, 0.0};
		for (int q = 0; q < nuau[i]; q++) {
			const int a = a0 + q;
			if (q > 0)
				for (int k = 0; k < 3; k++) prev[k] += ora_wrap(x[3 * a + k] - x[3 * (a - 1) + k], L[k]);
			for (int k = 0; k < 3; k++) c[k] += m[a] * prev[k];
		}
		for (int k = 0; k < 3; k++) {
			double v = c[k] / mmol[i];
			if (v > L[k]) v -= L[k];
			else if (v < 0.0) v += L[k];
			cm[3 * i + k] = v;
		}
	}
}

void ora_mol_velcm(int nmol, const int *start, const int *atoms, const double *mmol, const double *v,
		   const double *m, double *vcm)
{
	for (int i = 0; i < nmol; i++) {
		double s[3] = {0.0, 0.0, 0.0};
		for (int q = start[i]; q < start[i + 1]; q++)
			for (int k = 0; k < 3; k++) s[k] += v[3 * atoms[q] + k] * m[atoms[q]];
		for (int k = 0; k < 3; k++) vcm[3 * i + k] = s[k] / mmol[i];
	}
}

/* kin_P_mol = sum M v v^T; pot_P_mol = sum_{i<j} F[i][j] (x) R_ij with R_ij
 * the minimum image of cm_i - cm_j (row-major 3x3 each) */
void ora_mol_pressure(int nmol, const double *F, const double *cm, const double *vcm,
		      const double *mmol, const double L[3], double *kinP, double *potP)
{
	for (int q = 0; q < 9; q++) kinP[q] = potP[q] = 0.0;
	for (int i = 0; i < nmol; i++)
		for (int k = 0; k < 3; k++)
			for (int kk = 0; kk < 3; kk++) kinP[3 * k + kk] += mmol[i] * vcm[3 * i + k] * vcm[3 * i + kk];
	for (int i = 0; i < nmol - 1; i++)
		for (int j = i + 1; j < nmol; j++) {
			double r[3];
			for (int k = 0; k < 3; k++) r[k] = ora_wrap(cm[3 * i + k] - cm[3 * j + k], L[k]);
			const double *f = F + ((long)i * nmol + j) * 3;
			for (int k = 0; k < 3; k++)
				for (int kk = 0; kk < 3; kk++) potP[3 * k + kk] += f[k] * r[kk];
		}
}
