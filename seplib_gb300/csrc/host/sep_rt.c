/*
 * sep_rt.c - host runtime: contexts, residency, deferred pair passes and the
 * ordered application of accumulator slots to sepret (see sep_rt.h).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "sep_rt.h"

#define RT_MAXCTX 256

static rt_ctx *g_ctx[RT_MAXCTX];
char rt_errbuf[512];

void rt_check(int rc, const char *what)
{
	if (rc == SEPDEV_OK) return;
	snprintf(rt_errbuf, sizeof rt_errbuf, "%s failed (%d): %s", what, rc, sepdev_last_error());
	sep_error("%s", rt_errbuf);
}

rt_ctx *rt_find(const seppart *ptr)
{
	for (int k = 0; k < RT_MAXCTX; k++)
		if (g_ctx[k] && g_ctx[k]->ptr == ptr) return g_ctx[k];
	return NULL;
}

rt_ctx *rt_get(seppart *ptr, const char *caller)
{
	rt_ctx *c = rt_find(ptr);
	if (!c) sep_error("%s: particle array was not allocated by sep_init", caller);
	return c;
}

/* k-th registry entry (NULL when free), (rt_ctx *)-1 past the end */
rt_ctx *rt_each(int k)
{
	if (k < 0 || k >= RT_MAXCTX) return (rt_ctx *)-1;
	return g_ctx[k];
}

rt_ctx *rt_register(seppart *ptr, long n)
{
	for (int k = 0; k < RT_MAXCTX; k++)
		if (!g_ctx[k]) {
			rt_ctx *c = calloc(1, sizeof(rt_ctx));
			if (!c) sep_error("sep_init: couldn't allocate memory");
			c->ptr = ptr;
			c->n = n;
			c->host_valid = 1;
			c->list_stale = 1;
			c->pass_slot = -1;
			c->forces_zero = 0;
			c->seed = RT_SEED_DEFAULT;
			g_ctx[k] = c;
			return c;
		}
	sep_error("sep_init: too many particle arrays alive (%d)", RT_MAXCTX);
	return NULL;
}

void rt_unregister(seppart *ptr)
{
	for (int k = 0; k < RT_MAXCTX; k++)
		if (g_ctx[k] && g_ctx[k]->ptr == ptr) {
			rt_mv_drop(g_ctx[k]);
			if (g_ctx[k]->dev) sepdev_destroy(g_ctx[k]->dev);
			free(g_ctx[k]);
			g_ctx[k] = NULL;
		}
}

/* ---- upload / download ---------------------------------------------------- */

static int type_id(rt_ctx *c, char t)
{
	for (int k = 0; k < c->ntypes; k++)
		if (c->tchar[k] == t) return k;
	if (c->ntypes == SEPDEV_MAXTYPES)
		sep_error("more than %d particle types are not supported on the GPU", SEPDEV_MAXTYPES);
	c->tchar[c->ntypes] = t;
	return c->ntypes++;
}

int rt_type_id(rt_ctx *c, char t)
{
	for (int k = 0; k < c->ntypes; k++)
		if (c->tchar[k] == t) return k;
	return -1;
}

/* pv, pa, prevf, randn and ldiff of the seppart records to the device */
static void ext_upload(rt_ctx *c)
{
	const long n = c->n;
	const seppart *p = c->ptr;
	double *buf = malloc(sizeof(double) * 13 * n);
	if (!buf) sep_error("couldn't allocate memory");
	double *pv = buf, *pa = buf + 3 * n, *pf = buf + 6 * n, *rn = buf + 9 * n, *ld = buf + 12 * n;
	for (long i = 0; i < n; i++) {
		for (int k = 0; k < 3; k++) {
			pv[3 * i + k] = p[i].pv[k];
			pa[3 * i + k] = p[i].pa[k];
			pf[3 * i + k] = p[i].prevf[k];
			rn[3 * i + k] = p[i].randn[k];
		}
		ld[i] = p[i].ldiff;
	}
	rt_check(sepdev_ext_enable(c->dev), "stochastic fields");
	rt_check(sepdev_ext_upload(c->dev, pv, pa, pf, rn, ld), "stochastic upload");
	free(buf);
}

static void ext_download(rt_ctx *c)
{
	const long n = c->n;
	seppart *p = c->ptr;
	double *buf = malloc(sizeof(double) * 12 * n);
	if (!buf) sep_error("couldn't allocate memory");
	double *pv = buf, *pa = buf + 3 * n, *pf = buf + 6 * n, *rn = buf + 9 * n;
	rt_check(sepdev_ext_download(c->dev, pv, pa, pf, rn), "stochastic download");
	for (long i = 0; i < n; i++)
		for (int k = 0; k < 3; k++) {
			p[i].pv[k] = pv[3 * i + k];
			p[i].pa[k] = pa[3 * i + k];
			p[i].prevf[k] = pf[3 * i + k];
			p[i].randn[k] = rn[3 * i + k];
		}
	free(buf);
}

void rt_need_ext(rt_ctx *c, const sepsys *sys)
{
	rt_need_device(c, sys);
	if (c->ext_on) return;
	c->ext_on = 1;
	ext_upload(c);
}

static void upload_topology(rt_ctx *c)
{
	const long n = c->n;
	seppart *p = c->ptr;
	/* exclusion CSR tables from the per-particle partner arrays */
	int *bs = calloc(n + 1, sizeof(int)), *as = calloc(n + 1, sizeof(int));
	if (!bs || !as) sep_error("couldn't allocate memory");
	for (long i = 0; i < n; i++) {
		int nb = 0, na = 0;
		for (int k = 0; k < SEP_BOND && p[i].bond[k] != -1; k++) nb++;
		na = nb;
		for (int k = 0; k < SEP_ANGLE && p[i].angle[k] != -1; k++) na++;
		for (int k = 0; k < SEP_DIHED && p[i].dihed[k] != -1; k++) na++;
		bs[i + 1] = bs[i] + nb;
		as[i + 1] = as[i] + na;
	}
	int *bi = malloc(sizeof(int) * (bs[n] + 1)), *ai = malloc(sizeof(int) * (as[n] + 1));
	if (!bi || !ai) sep_error("couldn't allocate memory");
	for (long i = 0; i < n; i++) {
		int q = bs[i], r = as[i];
		for (int k = 0; k < SEP_BOND && p[i].bond[k] != -1; k++) { bi[q++] = p[i].bond[k]; ai[r++] = p[i].bond[k]; }
		for (int k = 0; k < SEP_ANGLE && p[i].angle[k] != -1; k++) ai[r++] = p[i].angle[k];
		for (int k = 0; k < SEP_DIHED && p[i].dihed[k] != -1; k++) ai[r++] = p[i].dihed[k];
	}
	rt_check(sepdev_set_exclusions(c->dev, bs, bi, as, ai), "exclusion upload");
	free(bs); free(as); free(bi); free(ai);
	if (c->topo_sys && c->topo_sys->molptr) {
		sepmolinfo *m = c->topo_sys->molptr;
		rt_check(sepdev_set_topology(c->dev, m->flag_bonds ? (int)m->num_bonds : 0, m->blist,
					     m->flag_angles ? (int)m->num_angles : 0, m->alist,
					     m->flag_dihedrals ? (int)m->num_dihedrals : 0, m->dlist),
			 "topology upload");
		c->has_topo = 1;
	}
	c->topo_dirty = 0;
}

void rt_need_device(rt_ctx *c, const sepsys *sys)
{
	if (!c->dev) {
		if (sepdev_device_count() < 1)
			sep_error("no CUDA device is available; this sep library runs on the GPU only");
		rt_check(sepdev_create(&c->dev, c->n), "device context");
	}
	if (c->dev_valid && !c->topo_dirty) return;
	const int uploading = !c->dev_valid;
	if (!c->dev_valid && sepdev_direct_io(c->dev)) {
		/* the device reads the seppart records itself */
		double sv2 = 0.0, maxd2 = 0.0;
		int nt = 0;
		const int rc = sepdev_upload_parts(c->dev, c->ptr, sys->length, SEPDEV_MAXTYPES, c->tchar,
						   &nt, &sv2, &maxd2);
		if (rc == SEPDEV_EOVERFLOW)
			sep_error("more than %d particle types are not supported on the GPU", SEPDEV_MAXTYPES);
		rt_check(rc, "upload");
		c->ntypes = nt;
		c->dev_valid = 1;
		c->list_stale = 1;
		c->sumv2 = sv2;
		c->sumv2_valid = 1;
		c->pending_trigger = sqrt(maxd2) > 0.5 * sys->skin;
	}
	if (!c->dev_valid) {
		const long n = c->n;
		seppart *p = c->ptr;
		double *x = malloc(sizeof(double) * 3 * n), *v = malloc(sizeof(double) * 3 * n);
		double *f = malloc(sizeof(double) * 3 * n), *m = malloc(sizeof(double) * n);
		double *z = malloc(sizeof(double) * n);
		int *ty = malloc(sizeof(int) * n), *mol = malloc(sizeof(int) * n);
		int *cr = malloc(sizeof(int) * 3 * n), *cn = malloc(sizeof(int) * 3 * n);
		if (!x || !v || !f || !m || !z || !ty || !mol || !cr || !cn)
			sep_error("couldn't allocate memory");
		double sv2 = 0.0, maxd2 = 0.0;
		c->ntypes = 0;
		for (long i = 0; i < n; i++) {
			double d2 = 0.0;
			for (int k = 0; k < 3; k++) {
				x[3 * i + k] = p[i].x[k];
				v[3 * i + k] = p[i].v[k];
				f[3 * i + k] = p[i].f[k];
				cr[3 * i + k] = p[i].crossings[k];
				cn[3 * i + k] = p[i].cross_neighb[k];
				sv2 += p[i].v[k] * p[i].v[k] * p[i].m;
				double r = p[i].x[k] - p[i].xn[k];
				const double L = sys->length[k];
				if (r > 0.5 * L) r -= L; else if (r < -0.5 * L) r += L;
				d2 += r * r;
			}
			if (d2 > maxd2) maxd2 = d2;
			m[i] = p[i].m;
			z[i] = p[i].z;
			ty[i] = type_id(c, p[i].type);
			mol[i] = p[i].molindex;
		}
		rt_check(sepdev_upload(c->dev, x, v, f, m, z, ty, mol, cr, cn, sys->length), "upload");
		free(x); free(v); free(f); free(m); free(z); free(ty); free(mol); free(cr); free(cn);
		c->dev_valid = 1;
		c->list_stale = 1;
		c->sumv2 = sv2;
		c->sumv2_valid = 1;
		/* The reference measures displacements from xn, which sep_init leaves
		 * unset; the device measures from the positions of its own list
		 * builds.  When the host xn is already more than skin/2 away, the
		 * reference's next leap-frog reports an update, so ours does too. */
		c->pending_trigger = sqrt(maxd2) > 0.5 * sys->skin;
	}
	if (uploading && c->ext_on) ext_upload(c);
	if (c->mv_on && !c->mv_uploaded) {
		rt_check(sepdev_molvir_enable(c->dev, c->mv_nmol, c->mv_first, c->mv_nuau, c->mv_start,
					      c->mv_atoms, c->mv_mass), "molecular tables");
		c->mv_uploaded = 1;
	}
	if (c->topo_dirty) upload_topology(c);
}

rt_ctx *rt_find_molinfo(const sepmolinfo *m)
{
	for (int k = 0; k < RT_MAXCTX; k++)
		if (g_ctx[k] && g_ctx[k]->mv_on && g_ctx[k]->mv_info == m) return g_ctx[k];
	return NULL;
}

void rt_mv_drop(rt_ctx *c)
{
	free(c->mv_first); free(c->mv_nuau); free(c->mv_start); free(c->mv_atoms); free(c->mv_mass);
	c->mv_first = c->mv_nuau = c->mv_start = c->mv_atoms = NULL;
	c->mv_mass = NULL;
	c->mv_on = c->mv_uploaded = 0;
	c->mv_info = NULL;
	if (c->bm_tab) sepdev_moltab_destroy(c->bm_tab);
	c->bm_tab = NULL;
	c->bm_mols = NULL;
	if (c->dev) sepdev_molvir_disable(c->dev);
}

/* bond lengths, angles and dihedral angles of the last bonded calls */
static void term_values_to_host(rt_ctx *c)
{
	if (c->has_topo && c->topo_sys && c->topo_sys->molptr) {
		sepmolinfo *m = c->topo_sys->molptr;
		if (m->flag_bonds && m->blengths) sepdev_term_values(c->dev, 0, m->blengths);
		if (m->flag_angles && m->angles) sepdev_term_values(c->dev, 1, m->angles);
		if (m->flag_dihedrals && m->dihedrals) sepdev_term_values(c->dev, 2, m->dihedrals);
	}
}

void rt_need_host(rt_ctx *c)
{
	if (c->host_valid) return;
	rt_flush(c);
	if (sepdev_direct_io(c->dev)) {
		/* the device writes the seppart records itself */
		rt_check(sepdev_download_parts(c->dev, c->ptr, c->forces_zero), "download");
		term_values_to_host(c);
		if (c->ext_on) ext_download(c);
		c->host_valid = 1;
		return;
	}
	const long n = c->n;
	seppart *p = c->ptr;
	double *x = malloc(sizeof(double) * 3 * n), *v = malloc(sizeof(double) * 3 * n);
	double *f = malloc(sizeof(double) * 3 * n), *xn = malloc(sizeof(double) * 3 * n);
	int *cr = malloc(sizeof(int) * 3 * n), *cn = malloc(sizeof(int) * 3 * n);
	if (!x || !v || !f || !xn || !cr || !cn) sep_error("couldn't allocate memory");
	rt_check(sepdev_download(c->dev, x, v, f, cr, cn, xn), "download");
	for (long i = 0; i < n; i++)
		for (int k = 0; k < 3; k++) {
			p[i].x[k] = x[3 * i + k];
			p[i].v[k] = v[3 * i + k];
			p[i].f[k] = c->forces_zero ? 0.0 : f[3 * i + k];
			p[i].a[k] = p[i].f[k] / p[i].m;
			p[i].crossings[k] = cr[3 * i + k];
			p[i].cross_neighb[k] = cn[3 * i + k];
			p[i].xn[k] = xn[3 * i + k];
		}
	free(x); free(v); free(f); free(xn); free(cr); free(cn);
	term_values_to_host(c);
	if (c->ext_on) ext_download(c);
	c->host_valid = 1;
}

void rt_host_modified(rt_ctx *c)
{
	rt_need_host(c);
	c->dev_valid = 0;
	c->x0_valid = 0;
	c->forces_zero = 0;
}

/* ---- slots and operations ------------------------------------------------------ */

int rt_new_slot(rt_ctx *c)
{
	if (c->nslots >= 15) rt_flush(c);
	return c->nslots++;
}

void rt_add_op(rt_ctx *c, sepret *ret, int kind, int slot, int chan)
{
	if (c->nops == RT_MAXOPS) rt_flush(c);
	rt_op *o = &c->ops[c->nops++];
	o->ret = ret; o->kind = kind; o->slot = slot; o->chan = chan;
}

int rt_ret_pending(rt_ctx *c, const sepret *ret)
{
	for (int k = 0; k < c->nops; k++)
		if (c->ops[k].ret == ret) return 1;
	return 0;
}

static void add_sym(double P[3][3], const double *s, double w)
{
	P[0][0] += w * s[0]; P[0][1] += w * s[1]; P[0][2] += w * s[2];
	P[1][0] += w * s[1]; P[1][1] += w * s[3]; P[1][2] += w * s[4];
	P[2][0] += w * s[2]; P[2][1] += w * s[4]; P[2][2] += w * s[5];
}

/* Build the device pair table from the pending terms. */
void rt_pairset(rt_ctx *c, sepdev_pairset *ps)
{
	memset(ps, 0, sizeof *ps);
	ps->ntypes = c->ntypes > 0 ? c->ntypes : 1;
	ps->nchan = c->nterms;
	for (int t = 0; t < c->nterms; t++) {
		const rt_term *T = &c->terms[t];
		for (int a = 0; a < c->ntypes; a++)
			for (int b = 0; b < c->ntypes; b++) {
				const char ca = c->tchar[a], cb = c->tchar[b];
				if (!((ca == T->t0 && cb == T->t1) || (ca == T->t1 && cb == T->t0))) continue;
				sepdev_pot *P = &ps->pot[a * ps->ntypes + b];
				P->kind = T->kind;
				P->chan = t;
				P->rc2 = (float)(T->rc * T->rc);
				P->eps48 = (float)(48.0 * T->eps);
				P->eps4 = (float)(4.0 * T->eps);
				P->sig2 = (float)(T->sigma * T->sigma);
				P->aw = (float)T->aw;
				P->awh = (float)(0.5 * T->aw);
				P->ushift = (float)T->ushift;
				P->ushl = (float)(T->ushift - (double)P->ushift);
				P->table = T->table;
			}
	}
	if (c->coul_on) {
		ps->coulomb = 1;
		ps->coul_rc = (float)c->coul_cf;
		ps->coul_rc2 = (float)(c->coul_cf * c->coul_cf);
		ps->coul_irc2 = (float)(1.0 / (c->coul_cf * c->coul_cf));
		ps->coul_irc = (float)(1.0 / c->coul_cf);
	}
}

static int pass_pending(const rt_ctx *c) { return c->pass_slot >= 0; }

static void clear_pass(rt_ctx *c)
{
	c->nterms = 0;
	c->coul_on = 0;
	c->pass_slot = -1;
}

void rt_open_pass(rt_ctx *c, sepret *ret)
{
	/* both slots of a pass come from one flush window */
	if (c->nslots >= 14) rt_flush(c);
	c->pass_slot = rt_new_slot(c);
	rt_add_op(c, ret, OP_VIRIAL, c->pass_slot, 0);
	c->mv_slot = -1;
	if (c->mv_on) {
		c->mv_slot = rt_new_slot(c);
		rt_add_op(c, NULL, OP_MOLVIR, c->mv_slot, 0);
	}
}

/* the device writes the next pass's molecular sums to the pass's own slot */
void rt_pass_mol_slot(rt_ctx *c)
{
	if (c->mv_on && c->mv_uploaded)
		rt_check(sepdev_molvir_slot(c->dev, c->mv_slot), "molecular slot");
}

void rt_launch_pass(rt_ctx *c)
{
	if (!pass_pending(c)) return;
	sepdev_pairset ps;
	rt_pairset(c, &ps);
	rt_pass_mol_slot(c);
	rt_check(sepdev_pair_forces(c->dev, &ps, !c->forces_zero, c->pass_slot), "pair forces");
	c->forces_zero = 0;
	clear_pass(c);
}

/* Bonded calls are evaluated together: the terms of one kind each that are
 * pending go to one launch when the forces are next needed.  A second term
 * of a kind already pending launches the batch first. */
void rt_queue_bonded(rt_ctx *c, const sepdev_bterm *t)
{
	for (int k = 0; k < c->nbq; k++)
		if (c->bq[k].kind == t->kind) {
			rt_launch_bonded(c);
			break;
		}
	c->bq[c->nbq++] = *t;
}

void rt_launch_bonded(rt_ctx *c)
{
	if (c->nbq == 0) return;
	rt_check(sepdev_bonded(c->dev, c->bq, c->nbq, !c->forces_zero), "bonded forces");
	c->forces_zero = 0;
	c->nbq = 0;
}

void rt_materialize_forces(rt_ctx *c)
{
	if (pass_pending(c)) rt_launch_pass(c);
	rt_launch_bonded(c);
	if (c->forces_zero) {
		rt_check(sepdev_zero_forces(c->dev), "force reset");
		c->forces_zero = 0;
	}
	if (c->friction) {
		rt_check(sepdev_friction(c->dev, c->friction_alpha), "friction");
		c->friction = 0;
		c->friction_alpha = 0.0;
	}
}

static int read_slots(rt_ctx *c, sepsys *sys, int lf_slot, int step_may_skip)
{
	if (!c->dev) return 0;
	double vals[16 * SLOT_FIELDS];
	unsigned flags[4];
	/* the read-back clears the slots, except after a deferred step on a
	 * list whose build overflowed: that step did nothing, and the slots and
	 * the operations stay for its second run */
	rt_check(sepdev_slots_take(c->dev, c->nslots, vals, flags, step_may_skip), "slot read-back");
	if (step_may_skip && (flags[0] & 1u)) return 1;
	for (int k = 0; k < c->nops; k++) {
		const rt_op *o = &c->ops[k];
		const double *s = vals + o->slot * SLOT_FIELDS;
		sepret *r = o->ret;
		switch (o->kind) {
		case OP_PAIR_ASSIGN: r->epot = s[SLOT_EPOT0 + o->chan]; break;
		case OP_PAIR_ADD: r->epot += s[SLOT_EPOT0 + o->chan]; break;
		case OP_VIRIAL: add_sym(r->pot_P, s + SLOT_POTP, 1.0); break;
		case OP_COUL: r->epot += s[SLOT_ECOUL]; r->ecoul += s[SLOT_ECOUL]; break;
		case OP_BOND:
			r->epot += s[SLOT_EPOT0];
			add_sym(r->pot_P, s + SLOT_POTP, 1.0);
			add_sym(r->pot_P_bond, s + SLOT_POTPB, 1.0);
			break;
		case OP_EADD: r->epot += s[SLOT_EPOT0]; break;
		case OP_MOLVIR:
			for (int q = 0; q < 9; q++) {
				c->molW[q] += s[q];
				c->molN[q] += s[9 + q];
			}
			break;
		case OP_DPD_VIR:
			add_sym(r->pot_P, s + SLOT_POTP, 1.0);
			add_sym(r->pot_P_conservative, s + SLOT_POTP, 1.0);
			add_sym(r->pot_P_random, s + SLOT_POTPB, 1.0);
			add_sym(r->pot_P_dissipative, vals + o->chan * SLOT_FIELDS + SLOT_POTP, 1.0);
			break;
		case OP_KIN:
			r->ekin += 0.5 * s[SLOT_EKIN];
			add_sym(r->kin_P, s + SLOT_KINP, 1.0);
			break;
		}
	}
	if (lf_slot >= 0) {
		const double *s = vals + lf_slot * SLOT_FIELDS;
		c->sumv2 = s[SLOT_SUMV2];
		c->sumv2_valid = 1;
		if (sys) {
			const double md = s[SLOT_MAXD2];
			if (md > sys->max_dist2) sys->max_dist2 = md;
		}
	}
	c->nops = 0;
	c->nslots = 0;
	return 0;
}

void rt_read_slots(rt_ctx *c, sepsys *sys, int lf_slot)
{
	read_slots(c, sys, lf_slot, 0);
}

int rt_read_step_slots(rt_ctx *c, sepsys *sys, int lf_slot)
{
	return read_slots(c, sys, lf_slot, 1);
}

void rt_flush(rt_ctx *c)
{
	if (!c->dev) return;
	rt_materialize_forces(c);
	if (c->nops || c->nslots) rt_read_slots(c, NULL, -1);
}

/* ---- neighbour list ------------------------------------------------------------ */

/* Exclusion mode of a pair-force call under the system's update method: the
 * O(N^2) paths exclude direct bonds only (source/sepprfrc.c:35 and :317), the
 * linked-cell builder excludes bond, angle and dihedral partners (:582). */
static int excl_mode(unsigned update, unsigned opt, int brute_excl_bonds)
{
	if (opt == SEP_EXCL_SAME_MOL) return SEPDEV_EXCL_SAMEMOL;
	if (opt == SEP_EXCL_BONDED) {
		if (update == SEP_LLIST_NEIGHBLIST) return SEPDEV_EXCL_ALLBONDED;
		return brute_excl_bonds ? SEPDEV_EXCL_BONDS : SEPDEV_EXCL_ALLBONDED;
	}
	return SEPDEV_EXCL_NONE;
}

void rt_prepare_list(rt_ctx *c, sepsys *sys, unsigned opt, int brute_excl_bonds)
{
	int want_excl = c->list_excl;
	double cfmax = sys->cf;
	if (sys->neighb_update == SEP_BRUTE) {
		/* no list in the reference: every call applies its own exclusions */
		want_excl = excl_mode(SEP_BRUTE, opt, brute_excl_bonds);
		if (c->brute_cf > cfmax) cfmax = c->brute_cf;
		if (want_excl != c->list_excl) c->list_stale = 1;
	} else if (sys->neighb_flag == 1) {
		want_excl = excl_mode(sys->neighb_update, opt, brute_excl_bonds);
		c->list_stale = 1;
		sys->neighb_flag = 0;
	} else if (c->list_stale) {
		/* first build, or the device state was re-uploaded */
		if (c->nbuild == 0) want_excl = excl_mode(sys->neighb_update, opt, brute_excl_bonds);
	}
	const double rlist = cfmax + sys->skin;
	if (rlist != c->list_rlist) c->list_stale = 1;
	if (!c->list_stale) return;
	/* the pending pass was meant for the old list */
	if (pass_pending(c)) rt_launch_pass(c);
	rt_launch_bonded(c);
	if (want_excl != SEPDEV_EXCL_NONE && want_excl != SEPDEV_EXCL_SAMEMOL && c->topo_dirty)
		rt_need_device(c, sys);
	/* the capacity check is left to the step's read-back, or to the next
	 * other consumer of the list (sepdev_build_list_deferred) */
	rt_check(sepdev_build_list_deferred(c->dev, rlist, want_excl, c->trigger_next),
		 "neighbour-list build");
	c->list_excl = want_excl;
	c->list_rlist = rlist;
	c->list_stale = 0;
	c->trigger_next = 0;
	c->nbuild++;
}
