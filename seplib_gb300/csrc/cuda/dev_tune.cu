// dev_tune.cu - the table of kernel parameters by system size (team size,
// neighbour groups per iteration, cell edge of the list build) that the
// autotuner (seplib_gb300/tune.py) fills from timed trials.  Host code only:
// the kernels take their parameters from the context or the batch.
#include <string.h>
#include "dev_common.cuh"

static sepdev_tuning g_tune = {1, {0}, {1}, {2}, {1.0}};

extern "C" int sepdev_tuning_set(const sepdev_tuning *t)
{
	if (!t || t->nclass < 1 || t->nclass > SEPDEV_NCLASS) return SEPDEV_EINVAL;
	for (int k = 0; k < t->nclass; k++) {
		if (t->team[k] != 1 && t->team[k] != 2) return SEPDEV_EINVAL;
		if (t->groups[k] != 1 && t->groups[k] != 2) return SEPDEV_EINVAL;
		if (!(t->cellf[k] >= 1.0 && t->cellf[k] <= 2.0)) return SEPDEV_EINVAL;
		if (k > 0 && k < t->nclass - 1 && t->nmax[k] <= t->nmax[k - 1]) return SEPDEV_EINVAL;
	}
	g_tune = *t;
	return SEPDEV_OK;
}

extern "C" void sepdev_tuning_get(sepdev_tuning *t)
{
	if (t) *t = g_tune;
}

extern "C" void sepdev_tuning_for(long n, int *team, int *groups, double *cellf)
{
	int k = 0;
	while (k < g_tune.nclass - 1 && n > g_tune.nmax[k]) k++;
	if (team) *team = g_tune.team[k];
	if (groups) *groups = g_tune.groups[k];
	if (cellf) *cellf = g_tune.cellf[k];
}
