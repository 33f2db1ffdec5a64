/*
 * sepdef.h - interface constants of the sep C API (GB300 implementation).
 *
 * The names and values below are part of the programming interface that
 * seplib programs compile against, so they are kept identical to the
 * reference's include/sepdef.h:19-64.  Only the constants a program or the
 * hot path uses are defined.
 */
#ifndef SEP_GB300_SEPDEF_H
#define SEP_GB300_SEPDEF_H

#define SEP_FALSE 0
#define SEP_TRUE  1

/* per-particle exclusion slots (bond / angle / dihedral partners) */
#define SEP_BOND  10
#define SEP_ANGLE 10
#define SEP_DIHED 20

/* neighbour-list capacity arguments accepted by sep_init() */
#define SEP_NEIGHB      3000
#define SEP_NUM_NEIGHB  3000
#define SEP_NO_NEIGHB   0

/* exclusion options for the pair-force and Coulomb calls */
#define SEP_NEIGHB_ALL            1
#define SEP_ALL                   1
#define SEP_NEIGHB_EXCL_BONDED    2
#define SEP_EXCL_BONDED           2
#define SEP_NEIGHB_EXCL_SAME_MOL  3
#define SEP_EXCL_SAME_MOL         3

#define SEP_MAX_NUM_MOL 10000

#define SEP_PI    3.14159265358979
#define SEP_WCACF 1.12246204830937
/* energy shift of the unit LJ potential at r = 2.5: -4(2.5^-12 - 2.5^-6) */
#define SEP_LJCF2 0.016316891136

#define SEP_MAXNID     100000
#define SEP_NRETVALS   10

/* force-calculation algorithm passed to sep_sys_setup() */
#define SEP_BRUTE             0
#define SEP_NEIGHBLIST        1
#define SEP_LLIST_NEIGHBLIST  2

#define SEP_LEAPFROG    0
#define SEP_NOSEHOOVER  1
#define SEP_ANDERSEN    2
#define SEP_SHAKE       3

/* the reference returns the same value for both outcomes */
#define SEP_SUCCESS 1
#define SEP_FAILURE 1

#endif
