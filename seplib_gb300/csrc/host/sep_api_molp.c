/*
 * sep_api_molp.c - molecular pressure tensor and molecular centres of mass
 * of the sep C API (reference source/sepret.c:85-102,
 * source/sepmol.c:683-748, :913-959).
 */
#include <math.h>
#include <stdlib.h>
#include "sep_rt.h"

static double wrap1(double d, double L)
{
	if (d > 0.5 * L) return d - L;
	if (d < -0.5 * L) return d + L;
	return d;
}

/* source/sepmol.c:683-729, on the host copy of the particles */
void sep_mol_cm(seppart *ptr, sepmol *mol, sepsys *sys)
{
	rt_ctx *c = rt_find(ptr);
	if (c) rt_need_host(c);
	for (unsigned n = 0; n < sys->molptr->num_mols; n++) {
		const int i = mol[n].index[0];
		double prev[3] = {ptr[i].x[0], ptr[i].x[1], ptr[i].x[2]}, cm[3] = {0.0, 0.0, 0.0};
		for (unsigned m = 0; m < mol[n].nuau; m++) {
			if (m > 0)
				for (int k = 0; k < 3; k++)
					prev[k] += wrap1(ptr[i + m].x[k] - ptr[i + m - 1].x[k], sys->length[k]);
			for (int k = 0; k < 3; k++) cm[k] += ptr[i + m].m * prev[k];
		}
		for (int k = 0; k < 3; k++) {
			double v = cm[k] / mol[n].m;
			if (v > sys->length[k]) v -= sys->length[k];
			else if (v < 0.0) v += sys->length[k];
			mol[n].x[k] = v;
		}
	}
}

/* source/sepmol.c:731-748 */
void sep_mol_velcm(seppart *atom, sepmol *mol, sepsys *sys)
{
	rt_ctx *c = rt_find(atom);
	if (c) rt_need_host(c);
	for (unsigned i = 0; i < sys->molptr->num_mols; i++) {
		for (int k = 0; k < 3; k++) mol[i].v[k] = 0.0;
		for (unsigned n = 0; n < mol[i].nuau; n++) {
			const int a = mol[i].index[n];
			for (int k = 0; k < 3; k++) mol[i].v[k] += atom[a].v[k] * atom[a].m;
		}
		for (int k = 0; k < 3; k++) mol[i].v[k] /= mol[i].m;
	}
}

void sep_mol_pressure_tensor(sepatom *atoms, sepmol *mols, sepret *ret, sepsys *sys)
{
	rt_ctx *c = rt_find_molinfo(sys->molptr);
	if (sys->molptr->flag_Fij == 1 && c && c->ptr == atoms) {
		rt_need_device(c, sys);
		rt_flush(c);
		const int nm = c->mv_nmol;
		double kin[9], corr[9], L0[3], L1[3];
		double *cv = malloc(sizeof(double) * 6 * (nm > 0 ? nm : 1));
		if (!cv) sep_error("%s: Couldn't allocate memory", __func__);
		rt_check(sepdev_mol_state(c->dev, kin, corr, cv, cv + 3 * nm, L0, L1), "molecular pressure");
		for (int i = 0; i < nm; i++)
			for (int k = 0; k < 3; k++) {
				mols[i].x[k] = cv[3 * i + k];
				mols[i].v[k] = cv[3 * nm + 3 * i + k];
			}
		free(cv);
		for (int k = 0; k < 3; k++)
			for (int kk = 0; kk < 3; kk++) {
				ret->kin_P_mol[k][kk] = kin[3 * k + kk];
				/* sum_{i<j} F_ij (x) R'_ij with R'_ij - R_ij = dR_i - dR_j
				 * - (L1 - L0) n_ij for the image n_ij of the pass */
				ret->pot_P_mol[k][kk] = c->molW[3 * k + kk] + corr[3 * k + kk] -
							(L1[kk] - L0[kk]) * c->molN[3 * k + kk];
			}
	}
	const double ivol = 1.0 / sys->volume;
	for (int k = 0; k < 3; k++)
		for (int kk = 0; kk < 3; kk++)
			ret->P_mol[k][kk] = (ret->kin_P_mol[k][kk] + ret->pot_P_mol[k][kk]) * ivol;
	ret->p_mol = (ret->P_mol[0][0] + ret->P_mol[1][1] + ret->P_mol[2][2]) / 3.0;
}
