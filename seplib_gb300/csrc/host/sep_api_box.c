/*
 * sep_api_box.c - box changes of the sep C API: compression
 * (sep_compress_box, sep_compress_box_dir, sep_compress_box_dir_length) and
 * the Berendsen barostats (sep_berendsen, sep_berendsen_iso,
 * sep_berendsen_mol), reference source/sepmisc.c:892-1084.  The box arithmetic and the sub-box grid
 * bookkeeping run on the host as in the reference; the positions are
 * rescaled on the device when it holds them.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include "sep_rt.h"

/* new edges L1, positions x_k *= sx[k] */
static void apply(seppart *ptr, sepsys *sys, const double L1[3], const double sx[3])
{
	rt_ctx *c = rt_find(ptr);
	if (c && c->dev && c->dev_valid) {
		/* pending pair terms belong to the old box */
		rt_materialize_forces(c);
		rt_check(sepdev_rescale_box(c->dev, L1, sx), "box change");
		c->host_valid = 0;
	} else {
		for (long n = 0; n < sys->npart; n++)
			for (int k = 0; k < 3; k++)
				if (sx[k] != 1.0) ptr[n].x[k] *= sx[k];
	}
	for (int k = 0; k < 3; k++) sys->length[k] = L1[k];
}

static void subbox(sepsys *sys, int k, double delta, const char *caller)
{
	if (sys->neighb_update == 0) return;
	sys->nsubbox[k] = sep_nsubbox(sys->cf, delta, sys->length[k]);
	if (sys->nsubbox[k] < 3)
		sep_warning("%s: Number of subboxes in x direction are less than three", caller);
	sys->lsubbox[k] = sys->length[k] / sys->nsubbox[k];
}

/* source/sepmisc.c:989-1024 */
void sep_compress_box(sepatom *ptr, double rhoD, double xi, sepsys *sys)
{
	const double density = sys->npart / sys->volume;
	if (fabs(density - rhoD) < 1e-6) return;
	if (density > rhoD) xi = 1.0 / xi;
	double L1[3], sx[3];
	for (int k = 0; k < 3; k++) {
		L1[k] = sys->length[k] * xi;
		sx[k] = xi;
		if (L1[k] < sys->cf * 2.0)
			sep_warning("%s: Box length too small compared to the maximum cut-off", __func__);
	}
	apply(ptr, sys, L1, sx);
	for (int k = 0; k < 3; k++) subbox(sys, k, sys->skin, __func__);
	sys->volume = sys->length[0] * sys->length[1] * sys->length[2];
}

/* one axis: edge times xi, positions times xi^(1/3) */
static void compress_axis(sepatom *ptr, double xi, int dir, sepsys *sys, const char *caller)
{
	double L1[3] = {sys->length[0], sys->length[1], sys->length[2]}, sx[3] = {1.0, 1.0, 1.0};
	L1[dir] *= xi;
	if (L1[dir] < sys->cf * 2.0)
		sep_warning("%s: Box length too small compared to the maximum cut-off", caller);
	sx[dir] = pow(xi, 1.0 / 3.0);
	apply(ptr, sys, L1, sx);
	subbox(sys, dir, 0.0, caller);
	sys->volume = sys->length[0] * sys->length[1] * sys->length[2];
}

/* source/sepmisc.c:1029-1054 */
void sep_compress_box_dir(sepatom *ptr, double rhoD, double xi, int dir, sepsys *sys)
{
	if (sys->npart / sys->volume < rhoD) compress_axis(ptr, xi, dir, sys, __func__);
}

/* source/sepmisc.c:1057-1082 */
void sep_compress_box_dir_length(sepatom *ptr, double length, double xi, int dir, sepsys *sys)
{
	if (sys->length[dir] > length) compress_axis(ptr, xi, dir, sys, __func__);
}

/* source/sepmisc.c:892-946: xi = 1 - beta dt (Pd - p) from the current
 * pressure; iso = 0 changes L_z only, iso = 1 all edges; positions are
 * scaled by xi^(1/3) on the same axes */
static void berendsen(sepatom *ptr, double Pd, double beta, sepret *ret, sepsys *sys, int iso)
{
	sep_pressure_tensor(ret, sys);
	const double xi = 1 - beta * sys->dt * (Pd - ret->p);
	const int k0 = iso ? 0 : 2;
	double L1[3] = {sys->length[0], sys->length[1], sys->length[2]}, sx[3] = {1.0, 1.0, 1.0};
	const double scale = pow(xi, 1.0 / 3.0);
	for (int k = k0; k < 3; k++) {
		L1[k] *= xi;
		sx[k] = scale;
	}
	apply(ptr, sys, L1, sx);
	sys->volume = sys->length[0] * sys->length[1] * sys->length[2];
	for (int k = k0; k < 3; k++) subbox(sys, k, 0.0, iso ? "sep_berendsen_iso" : "sep_berendsen");
}

void sep_berendsen(sepatom *ptr, double Pd, double beta, sepret *ret, sepsys *sys)
{
	berendsen(ptr, Pd, beta, ret, sys, 0);
}

void sep_berendsen_iso(sepatom *ptr, double Pd, double beta, sepret *ret, sepsys *sys)
{
	berendsen(ptr, Pd, beta, ret, sys, 1);
}

/* the device tables of a molecule array, kept while it stays the same */
static sepdev_moltab *berendsen_tables(rt_ctx *c, sepmol *mol, int nm)
{
	if (c->bm_tab && c->bm_mols == mol && c->bm_nmol == nm) return c->bm_tab;
	if (c->bm_tab) sepdev_moltab_destroy(c->bm_tab);
	c->bm_tab = NULL;
	int *first = malloc(sizeof(int) * nm), *nuau = malloc(sizeof(int) * nm);
	int *start = malloc(sizeof(int) * (nm + 1));
	double *mass = malloc(sizeof(double) * nm);
	if (!first || !nuau || !start || !mass) sep_error("%s: couldn't allocate memory", __func__);
	start[0] = 0;
	for (int m = 0; m < nm; m++) start[m + 1] = start[m] + (int)mol[m].nuau;
	int *atoms = malloc(sizeof(int) * (start[nm] > 0 ? start[nm] : 1));
	if (!atoms) sep_error("%s: couldn't allocate memory", __func__);
	for (int m = 0; m < nm; m++) {
		first[m] = mol[m].nuau > 0 ? mol[m].index[0] : 0;
		nuau[m] = (int)mol[m].nuau;
		mass[m] = mol[m].m;
		for (unsigned q = 0; q < mol[m].nuau; q++) atoms[start[m] + q] = mol[m].index[q];
	}
	rt_check(sepdev_moltab_create(c->dev, nm, first, nuau, start, atoms, mass, &c->bm_tab), "molecule tables");
	c->bm_mols = mol;
	c->bm_nmol = nm;
	free(first); free(nuau); free(start); free(atoms); free(mass);
	return c->bm_tab;
}

/* source/sepmisc.c:948-990 */
void sep_berendsen_mol(sepatom *ptr, sepmol *mol, double Pd, double beta, sepret *ret, sepsys *sys)
{
	const int nm = (int)sys->molptr->num_mols;
	/* reads the positions only (the reference takes the centres of mass
	 * first; the order does not matter) */
	sep_mol_pressure_tensor(ptr, mol, ret, sys);
	rt_ctx *c = rt_find(ptr);
	const int on_device = c && c->dev && c->dev_valid;
	double *dr0 = NULL;
	if (!on_device) {
		sep_mol_cm(ptr, mol, sys);
		dr0 = malloc(sizeof(double) * (sys->npart > 0 ? sys->npart : 1));
		if (!dr0) sep_error("%s: couldn't allocate memory", __func__);
		for (int n = 0; n < sys->npart; n++) {
			const int i = ptr[n].molindex;
			if (i != -1) dr0[n] = ptr[n].x[2] - mol[i].x[2];
		}
	}
	const double xi = 1 - beta * sys->dt * (Pd - ret->p_mol);
	const double L1 = sys->length[2] * xi;
	const double scale = pow(xi, 1.0 / 3.0);
	if (on_device) {
		/* pending pair terms belong to the old box */
		rt_materialize_forces(c);
		/* the program's centres of mass: set by the molecular pressure
		 * tensor when the molecular forces are on */
		if (sys->molptr->flag_Fij != 1) sep_mol_cm(ptr, mol, sys);
		rt_check(sepdev_berendsen_mol(c->dev, berendsen_tables(c, mol, nm), L1, scale), "molecular barostat");
		c->host_valid = 0;
		for (int n = 0; n < nm; n++) mol[n].x[2] *= scale;
	} else {
		for (int n = 0; n < nm; n++) mol[n].x[2] *= scale;
		for (int n = 0; n < sys->npart; n++) {
			const int i = ptr[n].molindex;
			if (i != -1) {
				double z = mol[i].x[2] + dr0[n];
				if (z > L1) z -= L1;
				else if (z < 0.0) z += L1;
				ptr[n].x[2] = z;
			}
		}
		free(dr0);
	}
	sys->length[2] = L1;
	sys->volume = sys->length[0] * sys->length[1] * sys->length[2];
	subbox(sys, 2, 0.0, __func__);
}
