/*
 * sep_api_force.c - pair forces, shifted-force Coulomb, bonded terms and the
 * topology reader of the sep C API.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "sep_rt.h"

/* ---- built-in potentials (source/sepmisc.c:115-182) ----------------------------- */

double sep_lj(double r2, char opt)
{
	const double ri = 1.0 / r2, ri3 = ri * ri * ri;
	if (opt == 'f') return 48.0 * ri3 * (ri3 - 0.5) * ri;
	if (opt == 'u') return 4.0 * ri3 * (ri3 - 1.0);
	return 0.0;
}

double sep_lj_shift(double r2, char opt)
{
	const double ri = 1.0 / r2, ri3 = ri * ri * ri;
	if (opt == 'f') return 48.0 * ri3 * (ri3 - 0.5) * ri;
	if (opt == 'u') return 4.0 * ri3 * (ri3 - 1.0) + SEP_LJCF2;
	return 0.0;
}

double sep_wca(double r2, char opt)
{
	const double ri = 1.0 / r2, ri3 = ri * ri * ri;
	if (opt == 'f') return 48.0 * ri3 * (ri3 - 0.5) * ri;
	if (opt == 'u') return 4.0 * ri3 * (ri3 - 1.0) + 1.0;
	return 0.0;
}

double sep_spring_x0(double r2, char opt)
{
	const double k = 500.0;
	if (opt == 'f') return -k;
	if (opt == 'u') return 0.5 * r2 * k;
	return 0.0;
}

/* ---- exclusion predicates (source/sepprfrc.c:703-740) ---------------------------- */

static unsigned share(const int *a, const int *b, int cap, int j1, int j2)
{
	for (int k = 0; k < cap; k++) {
		if (a[k] == -1 || b[k] == -1) break;
		if (a[k] == j2 || b[k] == j1) return 1;
	}
	return 0;
}

unsigned int sep_bond_share(seppart *p, int j1, int j2)
{
	return share(p[j1].bond, p[j2].bond, SEP_BOND, j1, j2);
}

unsigned int sep_angle_share(seppart *p, int j1, int j2)
{
	return share(p[j1].angle, p[j2].angle, SEP_ANGLE, j1, j2);
}

unsigned int sep_dihed_share(seppart *p, int j1, int j2)
{
	return share(p[j1].dihed, p[j2].dihed, SEP_DIHED, j1, j2);
}

unsigned int sep_bonded(seppart *p, int i, int j)
{
	return sep_bond_share(p, i, j) + sep_angle_share(p, i, j) + sep_dihed_share(p, i, j);
}

/* ---- pair terms ----------------------------------------------------------------------- */

#define TAB_POINTS 16384

/* A potential callback the device has no kernel for is tabulated on a
 * uniform r^2 grid from (cf/10)^2 to cf^2 and interpolated linearly. */
static int table_for(rt_ctx *c, double (*fun)(double, char), double cf)
{
	for (int t = 0; t < c->ntab; t++)
		if (c->tab_fun[t] == fun && c->tab_rc[t] == cf) return t;
	if (c->ntab == 4) sep_error("at most four tabulated pair potentials are supported");
	const double r2min = 0.01 * cf * cf, dr2 = (cf * cf - r2min) / (TAB_POINTS - 1);
	float *ft = malloc(sizeof(float) * TAB_POINTS), *u = malloc(sizeof(float) * TAB_POINTS);
	if (!ft || !u) sep_error("couldn't allocate memory");
	for (int k = 0; k < TAB_POINTS; k++) {
		const double r2 = r2min + k * dr2;
		ft[k] = (float)fun(r2, 'f');
		u[k] = (float)fun(r2, 'u');
	}
	const int t = c->ntab++;
	rt_check(sepdev_set_table(c->dev, t, TAB_POINTS, r2min, dr2, ft, u), "potential table");
	free(ft); free(u);
	c->tab_fun[t] = fun;
	c->tab_rc[t] = cf;
	return t;
}

static void term_from_fun(rt_ctx *c, rt_term *T, double (*fun)(double, char), double cf)
{
	memset(T, 0, sizeof *T);
	T->rc = cf;
	T->eps = 1.0; T->sigma = 1.0; T->aw = 1.0;
	if (fun == sep_lj_shift) { T->kind = SEPDEV_POT_LJ; T->ushift = SEP_LJCF2; }
	else if (fun == sep_lj) { T->kind = SEPDEV_POT_LJ; T->ushift = 0.0; }
	else if (fun == sep_wca) { T->kind = SEPDEV_POT_LJ; T->ushift = 1.0; }
	else { T->kind = SEPDEV_POT_TABLE; T->table = table_for(c, fun, cf); }
}

/* LJ with param = {cf, eps, sigma, aw}; the shift makes U(cf) = 0
 * (source/sepprfrc.c:785-786) */
static void term_from_param(rt_term *T, const double *p)
{
	memset(T, 0, sizeof *T);
	T->kind = SEPDEV_POT_LJ;
	T->rc = p[0]; T->eps = p[1]; T->sigma = p[2]; T->aw = p[3];
	T->ushift = -4.0 * p[1] * (pow(p[2] / p[0], 12.) - p[3] * pow(p[2] / p[0], 6.));
}

static int term_overlaps(const rt_ctx *c, const rt_term *T)
{
	for (int t = 0; t < c->nterms; t++) {
		const rt_term *U = &c->terms[t];
		if ((U->t0 == T->t0 && U->t1 == T->t1) || (U->t0 == T->t1 && U->t1 == T->t0)) return 1;
	}
	return 0;
}

/* append a pair term to the pending pass, opening one when needed */
static void add_term(rt_ctx *c, rt_term *T, const char *types, sepret *ret, int opkind)
{
	T->t0 = types[0];
	T->t1 = types[1];
	if (c->pass_slot >= 0 && (c->nterms == RT_MAXTERMS || term_overlaps(c, T))) rt_launch_pass(c);
	if (c->pass_slot < 0) rt_open_pass(c, ret);
	c->terms[c->nterms] = *T;
	rt_add_op(c, ret, opkind, c->pass_slot, c->nterms);
	c->nterms++;
	c->host_valid = 0;
}

static void brute_omp_reset(sepsys *sys)
{
	if (sys->neighb_update == SEP_BRUTE && sys->omp_flag) {
		sep_warning("omp flag set, SEP_BRUTE does not support threads.");
		sep_warning("Resetting omp flag");
		sys->omp_flag = false;
	}
}

/* source/sepprfrc.c:226-274 */
int sep_force_pairs(seppart *ptr, const char *types, double cf, double (*fun)(double, char),
		    sepsys *sys, sepret *retval, const unsigned opt)
{
	if (cf > sys->cf) sep_error("cutoff for an interaction cannot be larger than maximum cutoff");
	brute_omp_reset(sys);
	rt_ctx *c = rt_get(ptr, __func__);
	rt_need_device(c, sys);
	rt_prepare_list(c, sys, opt, 1);
	rt_term T;
	term_from_fun(c, &T, fun, cf);
	add_term(c, &T, types, retval, OP_PAIR_ASSIGN);
	return SEP_SUCCESS;
}

/* source/sepprfrc.c:743-780 */
void sep_force_lj(seppart *ptr, const char *types, const double *param, sepsys *sys,
		  sepret *retval, const unsigned opt)
{
	if (param[0] > sys->cf) sep_error("cutoff for an interaction cannot be larger than maximum cutoff");
	brute_omp_reset(sys);
	rt_ctx *c = rt_get(ptr, __func__);
	rt_need_device(c, sys);
	rt_prepare_list(c, sys, opt, 1);
	rt_term T;
	term_from_param(&T, param);
	add_term(c, &T, types, retval, OP_PAIR_ADD);
}

/* source/sepcoulomb.c:5-18: under SEP_BRUTE every pair within cf (with the
 * call's exclusions), otherwise the pairs of the current neighbour list */
void sep_coulomb_sf(seppart *ptr, double cf, sepsys *sys, sepret *retval, const unsigned opt)
{
	rt_ctx *c = rt_get(ptr, __func__);
	rt_need_device(c, sys);
	if (sys->neighb_update == SEP_BRUTE) {
		if (cf > c->brute_cf) c->brute_cf = cf;
		rt_prepare_list(c, sys, opt, 0);
	} else if (c->list_stale) {
		/* no device list yet: build one without consuming the update flag */
		const unsigned flag = sys->neighb_flag;
		sys->neighb_flag = 0;
		rt_prepare_list(c, sys, SEP_ALL, 1);
		sys->neighb_flag = flag;
	}
	if (c->pass_slot >= 0 && c->coul_on) rt_launch_pass(c);
	if (c->pass_slot < 0) rt_open_pass(c, retval);
	c->coul_on = 1;
	c->coul_cf = cf;
	rt_add_op(c, retval, OP_COUL, c->pass_slot, 0);
	c->host_valid = 0;
}

/* ---- bonded terms (source/sepmol.c:372-587) ---------------------------------------- */

/* The bonded calls are deferred: each takes its accumulator slot now and is
 * evaluated with the other pending bonded terms in one launch when the
 * forces are next needed (normally just before the leap-frog). */
static void bonded(seppart *ptr, sepsys *sys, const char *who, sepret *ret, int op,
		   sepdev_bterm *t)
{
	rt_ctx *c = rt_get(ptr, who);
	if (!c->topo_sys) c->topo_sys = sys;
	rt_need_device(c, sys);
	c->host_valid = 0;
	t->slot = rt_new_slot(c);
	rt_queue_bonded(c, t);
	rt_add_op(c, ret, op, t->slot, 0);
}

void sep_stretch_harmonic(sepatom *aptr, int type, const double lbond, const double ks,
			  sepsys *sys, sepret *ret)
{
	if (!sys->molptr->flag_bonds) return;
	sepdev_bterm t = {0};
	t.kind = 0; t.type = type; t.p0 = lbond; t.p1 = ks;
	bonded(aptr, sys, __func__, ret, OP_BOND, &t);
}

static void angles(seppart *ptr, int type, double angle0, double k, int cossq, sepsys *sys,
		   sepret *ret, const char *who)
{
	if (!sys->molptr->flag_angles) return;
	sepdev_bterm t = {0};
	t.kind = 1; t.type = type; t.p0 = angle0; t.p1 = k; t.cossq = cossq;
	bonded(ptr, sys, who, ret, OP_EADD, &t);
}

void sep_angle_harmonic(sepatom *ptr, int type, const double angle0, const double k,
			sepsys *sys, sepret *ret)
{
	angles(ptr, type, angle0, k, 0, sys, ret, __func__);
}

void sep_angle_cossq(sepatom *ptr, int type, const double angle0, const double k,
		     sepsys *sys, sepret *ret)
{
	angles(ptr, type, angle0, k, 1, sys, ret, __func__);
}

void sep_torsion_Ryckaert(sepatom *ptr, int type, const double g[6], sepsys *sys, sepret *ret)
{
	if (!sys->molptr->flag_dihedrals) return;
	sepdev_bterm t = {0};
	t.kind = 2; t.type = type;
	for (int k = 0; k < 6; k++) t.g[k] = g[k];
	bonded(ptr, sys, __func__, ret, OP_EADD, &t);
}

/* ---- topology reader (source/sepmol.c:5-369) ----------------------------------------
 * A section starts at a line that is exactly "[ name ]"; the line after it
 * is skipped (a comment in the reference's files); data lines follow until a
 * line starting with '[' or the end of the file. */

static FILE *open_section(const char *file, const char *name)
{
	FILE *fp = fopen(file, "r");
	if (!fp) sep_error("%s: Couldn't open file %s", __func__, file);
	char line[256], want[64];
	snprintf(want, sizeof want, "[ %s ]\n", name);
	while (fgets(line, sizeof line, fp))
		if (strcmp(line, want) == 0) {
			if (!fgets(line, sizeof line, fp)) sep_error("%s: Read error", __func__);
			return fp;
		}
	fclose(fp);
	return NULL;
}

/* next data line as nv unsigned values; 0 at the end of the section */
static int next_row(FILE *fp, unsigned *v, int nv)
{
	char line[256];
	while (fgets(line, sizeof line, fp)) {
		if (line[0] == '[') return 0;
		char *s = line;
		while (*s == ' ' || *s == '\t' || *s == '\r' || *s == '\n') s++;
		if (!*s) continue;
		int got = 0;
		char *end;
		for (int k = 0; k < nv; k++) {
			unsigned long x = strtoul(s, &end, 10);
			if (end == s) break;
			v[k] = (unsigned)x;
			s = end;
			got++;
		}
		if (got != nv) sep_error("sep_read_topology_file: Format in top file not correct");
		return 1;
	}
	return 0;
}

static void push_partner(int *arr, int cap, int who, const char *what)
{
	for (int k = 0; k < cap; k++)
		if (arr[k] == -1) { arr[k] = who; return; }
	sep_error("sep_read_topology_file: particle exceeds the allowed number of %s partners", what);
}

void sep_read_bonds_top(sepatom *ap, sepmolinfo *m, const char *file, int npart, char opt)
{
	m->flag_bonds = 1;
	m->num_bonds = 0; m->num_btypes = 0; m->num_mols = 0;
	m->blist = malloc(sizeof(unsigned)); m->blengths = malloc(sizeof(double));
	FILE *fp = open_section(file, "bonds");
	if (!fp) return;
	unsigned v[4];
	size_t cap = 0;
	while (next_row(fp, v, 4)) {
		if (v[1] >= (unsigned)npart || v[2] >= (unsigned)npart)
			sep_error("sep_read_topology_file: particle index out of range");
		if (m->num_bonds + 1 > cap) {
			cap = cap ? 2 * cap : 1024;
			m->blist = realloc(m->blist, sizeof(unsigned) * 3 * cap);
			if (!m->blist) sep_error("couldn't allocate memory");
		}
		unsigned *b = m->blist + 3 * m->num_bonds++;
		b[0] = v[1]; b[1] = v[2]; b[2] = v[3];
		ap[v[1]].molindex = (int)v[0];
		ap[v[2]].molindex = (int)v[0];
		push_partner(ap[v[1]].bond, SEP_BOND, (int)v[2], "bond");
		push_partner(ap[v[2]].bond, SEP_BOND, (int)v[1], "bond");
		if (v[3] > m->num_btypes) m->num_btypes = v[3];
		if (v[0] > m->num_mols) m->num_mols = v[0];
	}
	fclose(fp);
	m->num_btypes++;
	m->num_mols++;
	if (opt == 'v')
		printf("Succesfully read 'bond' section in file %s -> Found %d molecules, %d bond(s) and %d bond type(s).\n",
		       file, m->num_mols, m->num_bonds, m->num_btypes);
	m->blengths = realloc(m->blengths, sizeof(double) * (m->num_bonds + 1));
}

void sep_read_angles_top(sepatom *ap, sepmolinfo *m, const char *file, int npart, char opt)
{
	m->flag_angles = 1;
	m->num_angles = 0; m->num_atypes = 0;
	m->alist = malloc(sizeof(unsigned)); m->angles = malloc(sizeof(double));
	FILE *fp = open_section(file, "angles");
	if (!fp) return;
	unsigned v[5];
	size_t cap = 0;
	while (next_row(fp, v, 5)) {
		for (int k = 1; k < 4; k++)
			if (v[k] >= (unsigned)npart) sep_error("sep_read_topology_file: particle index out of range");
		if (m->num_angles + 1 > cap) {
			cap = cap ? 2 * cap : 1024;
			m->alist = realloc(m->alist, sizeof(unsigned) * 4 * cap);
			if (!m->alist) sep_error("couldn't allocate memory");
		}
		unsigned *a = m->alist + 4 * m->num_angles++;
		a[0] = v[1]; a[1] = v[2]; a[2] = v[3]; a[3] = v[4];
		const unsigned A = v[1], B = v[2], C = v[3];
		push_partner(ap[A].angle, SEP_ANGLE, B, "angle"); push_partner(ap[A].angle, SEP_ANGLE, C, "angle");
		push_partner(ap[B].angle, SEP_ANGLE, A, "angle"); push_partner(ap[B].angle, SEP_ANGLE, C, "angle");
		push_partner(ap[C].angle, SEP_ANGLE, A, "angle"); push_partner(ap[C].angle, SEP_ANGLE, B, "angle");
		if (v[4] > m->num_atypes) m->num_atypes = v[4];
	}
	fclose(fp);
	m->num_atypes++;
	if (opt == 'v')
		printf("Succesfully read 'angles' section in file %s -> Found %d angles(s) and %d bond angles(s).\n",
		       file, m->num_angles, m->num_atypes);
	m->angles = realloc(m->angles, sizeof(double) * (m->num_angles + 1));
}

void sep_read_dihedrals_top(sepatom *ap, sepmolinfo *m, const char *file, int npart, char opt)
{
	m->flag_dihedrals = 1;
	m->num_dihedrals = 0; m->num_dtypes = 0;
	m->dlist = malloc(sizeof(unsigned)); m->dihedrals = malloc(sizeof(double));
	FILE *fp = open_section(file, "dihedrals");
	if (!fp) return;
	unsigned v[6];
	size_t cap = 0;
	while (next_row(fp, v, 6)) {
		for (int k = 1; k < 5; k++)
			if (v[k] >= (unsigned)npart) sep_error("sep_read_topology_file: particle index out of range");
		if (m->num_dihedrals + 1 > cap) {
			cap = cap ? 2 * cap : 1024;
			m->dlist = realloc(m->dlist, sizeof(unsigned) * 5 * cap);
			if (!m->dlist) sep_error("couldn't allocate memory");
		}
		unsigned *d = m->dlist + 5 * m->num_dihedrals++;
		for (int k = 0; k < 5; k++) d[k] = v[k + 1];
		for (int r = 1; r < 5; r++)
			for (int q = 1; q < 5; q++)
				if (q != r) push_partner(ap[v[r]].dihed, SEP_DIHED, (int)v[q], "dihedral");
		if (v[5] > m->num_dtypes) m->num_dtypes = v[5];
	}
	fclose(fp);
	m->num_dtypes++;
	if (opt == 'v')
		printf("Succesfully read 'dihedrals' section in file %s -> Found %d dihedrals(s) and %d dihedral types(s).\n",
		       file, m->num_dihedrals, m->num_dtypes);
	m->dihedrals = realloc(m->dihedrals, sizeof(double) * (m->num_dihedrals + 1));
}

void sep_read_topology_file(sepatom *aptr, const char *file, sepsys *sys, char opt)
{
	rt_ctx *c = rt_get(aptr, __func__);
	rt_host_modified(c);
	sep_read_bonds_top(aptr, sys->molptr, file, (int)sys->npart, opt);
	sep_read_angles_top(aptr, sys->molptr, file, (int)sys->npart, opt);
	sep_read_dihedrals_top(aptr, sys->molptr, file, (int)sys->npart, opt);
	c->topo_sys = sys;
	c->topo_dirty = 1;
}

void sep_free_bonds(sepmolinfo *m)
{
	if (m && m->flag_bonds == 1) { free(m->blist); free(m->blengths); m->flag_bonds = 0; }
}

void sep_free_angles(sepmolinfo *m)
{
	if (m && m->flag_angles == 1) { free(m->alist); free(m->angles); m->flag_angles = 0; }
}

void sep_free_dihedrals(sepmolinfo *m)
{
	if (m && m->flag_dihedrals == 1) { free(m->dlist); free(m->dihedrals); m->flag_dihedrals = 0; }
}

/* molecule table (source/sepmol.c:590-658).  With at most SEP_MAX_NUM_MOL
 * molecules flag_Fij is set, as in the reference, and the molecular virial
 * is accumulated on the device (dev_molp.cu); the nmol^2 force matrix
 * itself is never formed, so molptr->Fij stays NULL. */
sepmol *sep_init_mol(sepatom *atom, sepsys *sys)
{
	rt_ctx *c = rt_get(atom, __func__);
	rt_need_host(c);
	const unsigned nm = sys->molptr->num_mols;
	int *cnt = calloc(nm + 1, sizeof(int));
	sepmol *mol = calloc(nm ? nm : 1, sizeof(sepmol));
	if (!cnt || !mol) sep_error("%s at %d: Couldn't allocate memory", __func__, __LINE__);
	for (long i = 0; i < sys->npart; i++)
		if (atom[i].molindex > -1 && (unsigned)atom[i].molindex < nm) cnt[atom[i].molindex]++;
	sys->molptr->max_nuau = 0;
	for (unsigned k = 0; k < nm; k++) {
		mol[k].nuau = cnt[k];
		mol[k].type = 'A';
		mol[k].index = malloc(sizeof(int) * (cnt[k] ? cnt[k] : 1));
		if (!mol[k].index) sep_error("%s: Couldn't allocate memory", __func__);
		if ((unsigned)cnt[k] > sys->molptr->max_nuau) sys->molptr->max_nuau = cnt[k];
		cnt[k] = 0;
	}
	for (long i = 0; i < sys->npart; i++) {
		const int a = atom[i].molindex;
		if (a > -1 && (unsigned)a < nm) {
			mol[a].index[cnt[a]++] = (int)i;
			mol[a].m += atom[i].m;
		}
	}
	free(cnt);
	sys->molptr->flag_Fij = 0;
	int ok = nm >= 1 && nm <= SEP_MAX_NUM_MOL;
	for (unsigned k = 0; k < nm && ok; k++)
		if (mol[k].nuau < 1 || mol[k].index[0] + (long)mol[k].nuau > sys->npart) ok = 0;
	if (!ok) {
		sep_warning("Molecular force/torque evaluation disabled");
		return mol;
	}
	rt_mv_drop(c);
	c->mv_nmol = (int)nm;
	c->mv_first = malloc(sizeof(int) * nm);
	c->mv_nuau = malloc(sizeof(int) * nm);
	c->mv_start = malloc(sizeof(int) * (nm + 1));
	c->mv_mass = malloc(sizeof(double) * nm);
	long tot = 0;
	for (unsigned k = 0; k < nm; k++) tot += mol[k].nuau;
	c->mv_atoms = malloc(sizeof(int) * (tot > 0 ? tot : 1));
	if (!c->mv_first || !c->mv_nuau || !c->mv_start || !c->mv_mass || !c->mv_atoms)
		sep_error("%s: Couldn't allocate memory", __func__);
	c->mv_start[0] = 0;
	for (unsigned k = 0; k < nm; k++) {
		c->mv_first[k] = mol[k].index[0];
		c->mv_nuau[k] = (int)mol[k].nuau;
		c->mv_mass[k] = mol[k].m;
		for (unsigned q = 0; q < mol[k].nuau; q++) c->mv_atoms[c->mv_start[k] + q] = mol[k].index[q];
		c->mv_start[k + 1] = c->mv_start[k] + (int)mol[k].nuau;
	}
	for (int q = 0; q < 9; q++) c->molW[q] = c->molN[q] = 0.0;
	c->mv_info = sys->molptr;
	c->mv_on = 1;
	c->mv_uploaded = 0;
	if (c->dev) {
		rt_flush(c);
		rt_check(sepdev_molvir_enable(c->dev, c->mv_nmol, c->mv_first, c->mv_nuau, c->mv_start,
					      c->mv_atoms, c->mv_mass), "molecular tables");
		c->mv_uploaded = 1;
	}
	sys->molptr->flag_Fij = 1;
	return mol;
}

void sep_free_mol(sepmol *mol, sepsys *sys)
{
	if (!mol) return;
	rt_ctx *c = rt_find_molinfo(sys->molptr);
	if (c) rt_mv_drop(c);
	sys->molptr->flag_Fij = 0;
	for (unsigned k = 0; k < sys->molptr->num_mols; k++) {
		free(mol[k].index);
		if (mol[k].shake_flag == 1) free(mol[k].blength);
	}
	free(mol);
}
