/*
 * A seplib program written against the sep C API only: an N=1000 NVT
 * Lennard-Jones run set up with the library's own lattice and seeded
 * velocities, linked-cell lists with skin 0.5.  It saves the initial state
 * (an observation point) and prints the final energies, the thermostat state
 * and the number of list updates, for the test to replay on the oracle.
 *
 *   usage: lj_loop <initial.xyz> <nsteps>
 */
#include <stdlib.h>
#include "sep.h"

int main(int argc, char **argv)
{
	if (argc != 3) sep_error("usage: lj_loop <initial.xyz> <nsteps>");
	const int natoms = 1000, nsteps = atoi(argv[2]);
	const double dens = 0.8442, dt = 0.005, temp = 1.0, tau = 10.0;
	const double lbox = pow(natoms / dens, 1.0 / 3.0);
	double alpha = 0.0;
	sepret ret;

	sepatom *atoms = sep_init(natoms, SEP_NEIGHB);
	sepsys sys = sep_sys_setup(lbox, lbox, lbox, 2.5, dt, natoms, SEP_LLIST_NEIGHBLIST);
	sep_set_lattice(atoms, sys);
	sep_set_vel_seed(atoms, temp, 42, sys);
	sep_set_skin(&sys, 0.5);
	sep_save_xyz(atoms, "A", argv[1], "w", &sys);

	for (int n = 0; n < nsteps; n++) {
		sep_reset_retval(&ret);
		sep_reset_force(atoms, &sys);
		sep_force_pairs(atoms, "AA", 2.5, sep_lj_shift, &sys, &ret, SEP_ALL);
		sep_nosehoover(atoms, temp, &alpha, tau, &sys);
		sep_leapfrog(atoms, &sys, &ret);
	}
	double mom = sep_eval_mom(atoms, natoms);
	sep_pressure_tensor(&ret, &sys);
	printf("%.17g %.17g %.17g %u %.17g %.17g %.17g\n", ret.epot, ret.ekin, alpha,
	       sys.nupdate_neighb, mom, ret.p, atoms[0].x[0]);
	sep_close(atoms, natoms);
	sep_free_sys(&sys);
	return 0;
}
