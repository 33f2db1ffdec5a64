/*
 * sepcoulomb.h - shifted-force Coulomb (reference include/sepcoulomb.h:39).
 */
#ifndef SEP_GB300_SEPCOULOMB_H
#define SEP_GB300_SEPCOULOMB_H

#include "sepdef.h"
#include "sepstrct.h"
#include "sepmisc.h"

/*
 * Shifted-force Coulomb between charged particles within cf:
 * F = zi zj (1/r^2 - 1/cf^2) r_vec/r, U = zi zj (1/r + (r - cf)/cf^2 - 1/cf).
 * With a neighbour list it reuses the list of the last pair-force call (so
 * `opt` only matters under SEP_BRUTE); energy is added to ret->epot and
 * ret->ecoul (reference :39, source/sepcoulomb.c:5-160).
 */
void sep_coulomb_sf(seppart *ptr, double cf, sepsys *sys, sepret *retval,
		    const unsigned opt);

#endif
