/*
 * sepstrct.h - data types of the sep C API (GB300 implementation).
 *
 * Programs read and write these structures directly (atoms[i].x, sys.npart,
 * ret.epot, ...), so every member, its type and its order follow the
 * reference's include/sepstrct.h:23-204.  Keeping the order also keeps the
 * byte layout: seppart is 568 bytes, sepsys 168 bytes and sepret 1000 bytes
 * on LP64, the same as the reference, so an object file compiled against the
 * reference headers links and runs against this library as well.
 *
 * On this implementation the particle state that the hot path changes
 * (x, v, f, a, crossings, cross_neighb, xn) lives on the GPU between calls;
 * the host copy in seppart is refreshed at the observation points listed in
 * sepgpu.h.  The device state is found from the seppart pointer itself, so
 * sepsys carries no extra member.
 */
#ifndef SEP_GB300_SEPSTRCT_H
#define SEP_GB300_SEPSTRCT_H

#include <stdbool.h>
#include "sepdef.h"

/* One particle (reference include/sepstrct.h:23-58). */
typedef struct {
	double x[3];          /* position, wrapped into [0, L) */
	double v[3];          /* velocity (leap-frog half step) */
	double f[3];          /* force */
	double a[3];          /* acceleration of the last integration step */
	double m;             /* mass */
	char type;            /* one-character particle type */
	double z;             /* point charge */

	int *neighb;          /* host neighbour list; unused here, lists live on the GPU */

	int cross_neighb[3];  /* box crossings since the last neighbour-list update */
	int crossings[3];     /* box crossings since the start */

	int molindex;         /* molecule index, -1 for a free particle */
	int bond[SEP_BOND];   /* bonded partners, -1 terminated */
	int angle[SEP_ANGLE]; /* partners through an angle, -1 terminated */
	int dihed[SEP_DIHED]; /* partners through a dihedral, -1 terminated */

	double sigma;         /* hard-sphere diameter */
	int *collid;          /* collision partners */
	double *colltime;     /* collision times */

	double ldiff;         /* Langevin diffusion coefficient */

	double xtrue[3];      /* unwrapped position */
	double x0[3];         /* initial position */
	double xn[3];         /* position at the last neighbour-list update */
	double xp[3];         /* previous position */
	double px[3];         /* predicted position */
	double pv[3];         /* predicted velocity */
	double pa[3];         /* predicted acceleration */
	double randn[3];      /* Gaussian random numbers */
	double prevf[3];      /* previous force */
} seppart;

typedef seppart sepatom;

/* Intramolecular topology (reference include/sepstrct.h:66-96). */
typedef struct {
	unsigned num_mols;
	unsigned max_nuau;

	int flag_bonds, flag_angles, flag_dihedrals;

	unsigned num_bonds;
	unsigned *blist;        /* (a, b, type) per bond */
	unsigned num_btypes;

	unsigned num_angles;
	unsigned *alist;        /* (a, b, c, type) per angle */
	unsigned num_atypes;

	unsigned num_dihedrals;
	unsigned *dlist;        /* (a, b, c, d, type) per dihedral */
	unsigned num_dtypes;

	double *blengths;       /* bond lengths of the last stretch call */
	double *angles;         /* angles of the last angle call */
	double *dihedrals;      /* dihedral angles of the last torsion call */

	unsigned flag_Fij;      /* molecular force matrix enabled */
	float ***Fij;           /* nmol x nmol x 3 */
	float ***Fiajb;         /* npart x nmol x 3 */
} sepmolinfo;

/* System description (reference include/sepstrct.h:103-135). */
typedef struct {
	long int npart;
	double length[3];
	double volume;

	int intgr_type;
	double dt;
	double tnow;
	unsigned ndof;
	double max_dist2;        /* largest squared displacement since the last update */

	double cf;               /* largest cut-off of the system */
	double lsubbox[3];
	int nsubbox[3];
	double skin;
	unsigned neighb_update;  /* SEP_BRUTE, SEP_NEIGHBLIST or SEP_LLIST_NEIGHBLIST */
	unsigned neighb_flag;    /* 1: the neighbour list must be rebuilt */
	unsigned nupdate_neighb; /* number of neighbour-list updates */

	bool omp_flag;
	unsigned int nthreads;

	int fun_cstate;

	sepmolinfo *molptr;
} sep3D;

typedef sep3D sepsys;

/* Molecule (reference include/sepstrct.h:140-167). */
typedef struct {
	double m;
	double x[3], xtrue[3];
	double v[3];

	unsigned nuau;
	int *index;

	double ete[3];
	double re2;
	double rg;
	double S[3];

	double s[3];
	double inertia[3][3];
	double w[3];
	int method_w;
	double pel[3];

	char type;

	unsigned nbonds;
	double *blength;
	int shake_flag;
} sepmol;

/* Return values (reference include/sepstrct.h:173-204). */
typedef struct {
	double etot;
	double ekin;
	double epot;
	double ecoul;
	double sumv2;

	double P[3][3];
	double kin_P[3][3];
	double pot_P[3][3];
	double p;

	double P_mol[3][3];
	double kin_P_mol[3][3];
	double pot_P_mol[3][3];
	double p_mol;

	double pot_P_conservative[3][3];
	double pot_P_random[3][3];
	double pot_P_dissipative[3][3];
	double pot_P_bond[3][3];

	double pot_T_mol[3][3];
	double kin_T_mol[3][3];
	double T_mol[3][3];
	double t_mol;
} sepret;

#endif
