// dev_noalloc.cu - Lennard-Jones forces without any device allocation.
//
// Some callers cannot call cudaMalloc: host applications that hand all device
// memory to their own pool allocator at start-up and allow no allocation
// outside it, and callers inside time-critical loops, where the implicit
// device-wide synchronisation of cudaMalloc and cudaFree would stall every
// step.  sep_gpu_lj_forces_noalloc serves them.  It computes the same forces
// and energy as sep_force_lj (shifted Lennard-Jones, parameters
// {cf, eps, sigma, aw}, reference source/sepprfrc.c:782-1000) from positions
// the caller already holds on the device, and writes them to device buffers
// the caller provides.  Its working memory (binned positions, cell counts and
// starts, the energy accumulator) is one fixed array in this file, so the
// call allocates nothing, in CUDA or elsewhere.
//
// Limits and sharing:
//  * at most NA_MAXN particles and NA_MAXC linked cells per call; larger
//    inputs are rejected with an error before any work is issued;
//  * the array is about 5 MB and every GPU that loads the library holds it
//    until the process exits;
//  * all calls share the one array, which keeps the previous call's contents:
//    each call clears what must start at zero itself, and calls that overlap
//    on the GPU (concurrent streams, or host threads) race on it;
//  * the cut-off may be at most half the shortest box side (the minimum
//    image of every pair within it is then unique); shorter boxes are
//    rejected;
//  * the first call on each device looks up the array's device address
//    (cudaGetSymbolAddress, with that device current) and caches it.  With
//    CUDA's lazy module loading (the default) that lookup is also what loads
//    this file's module onto the device, array included: the first call
//    takes the array's ~5 MB (plus the module's code) from the device, the
//    later calls take nothing.  Make that first call before the caller's
//    pool takes its memory and before any stream capture;
//  * particles join their cell through atomics, so the order in which a
//    particle's FP32 pair terms are summed varies from call to call: results
//    can differ between calls in the last bits (well inside FP32 rounding of
//    the pair maths).
#include <math.h>
#include <stdio.h>
#include "dev_common.cuh"

#define NA_MAXN (1 << 17)       // 131072 particles
#define NA_MAXC (1 << 16)       // 65536 cells
#define NA_MAXDEV 64

struct NaScratch {
	int4 pos[NA_MAXN];          // fixed-point high words + cell, caller order
	int slot[NA_MAXN];          // rank inside the cell
	int4 spos[NA_MAXN];         // cell order; .w = caller index
	int count[NA_MAXC];
	int start[NA_MAXC + 1];
	unsigned long long esum;    // energy, 64-bit fixed point (scale 2^32)
};

static __device__ __align__(256) NaScratch g_na_scratch;

static NaScratch *g_na_addr[NA_MAXDEV];

// clear the cell counts and the energy accumulator of the previous call
__global__ void k_na_clear(NaScratch *sc, int ncells)
{
	const int c = blockIdx.x * blockDim.x + threadIdx.x;
	if (c < ncells) sc->count[c] = 0;
	if (c == 0) sc->esum = 0ull;
}

__global__ void k_na_bin(NaScratch *sc, const double *__restrict__ x, int n, double ix0, double ix1,
			 double ix2, int nc0, int nc1, int nc2)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const double inv[3] = {ix0, ix1, ix2};
	unsigned h[3];
	for (int k = 0; k < 3; k++) {
		double fr = x[3 * i + k] * inv[k];
		fr -= floor(fr);
		double t = fr * 4294967296.0;
		h[k] = t >= 4294967296.0 ? 0u : (unsigned)t;
	}
	const int c = (int)__umulhi(h[0], (unsigned)nc0) +
		      nc0 * ((int)__umulhi(h[1], (unsigned)nc1) + nc1 * (int)__umulhi(h[2], (unsigned)nc2));
	sc->pos[i] = make_int4((int)h[0], (int)h[1], (int)h[2], c);
	sc->slot[i] = atomicAdd(&sc->count[c], 1);
}

// exclusive scan of the counts, one block
__global__ void k_na_scan(NaScratch *sc, int m)
{
	__shared__ int part[1024];
	const int chunk = (m + blockDim.x - 1) / blockDim.x;
	const int lo = threadIdx.x * chunk, hi = min(m, lo + chunk);
	int s = 0;
	for (int k = lo; k < hi; k++) s += sc->count[k];
	part[threadIdx.x] = s;
	__syncthreads();
	for (int off = 1; off < (int)blockDim.x; off <<= 1) {
		const int v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
		__syncthreads();
		part[threadIdx.x] += v;
		__syncthreads();
	}
	int run = threadIdx.x ? part[threadIdx.x - 1] : 0;
	for (int k = lo; k < hi; k++) { sc->start[k] = run; run += sc->count[k]; }
	if (threadIdx.x == blockDim.x - 1) sc->start[m] = part[threadIdx.x];
}

__global__ void k_na_scatter(NaScratch *sc, int n)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const int4 p = sc->pos[i];
	sc->spos[sc->start[p.w] + sc->slot[i]] = make_int4(p.x, p.y, p.z, i);
}

struct NaForceArgs {
	NaScratch *sc;
	int n;
	int nc[3];
	float fs[3];
	float rc2, sig2, eps48, eps4, awh, aw, ushift;
	double *f;
};

// one thread per particle (cell order): scan the 27 neighbouring cells
__global__ void __launch_bounds__(256) k_na_force(NaForceArgs a)
{
	const int s = blockIdx.x * blockDim.x + threadIdx.x;
	float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
	if (s < a.n) {
		const NaScratch *sc = a.sc;
		const int4 pi = sc->spos[s];
		const int cx = (int)__umulhi((unsigned)pi.x, (unsigned)a.nc[0]);
		const int cy = (int)__umulhi((unsigned)pi.y, (unsigned)a.nc[1]);
		const int cz = (int)__umulhi((unsigned)pi.z, (unsigned)a.nc[2]);
		// offsets -1..1, fewer when a side has two cells (no cell twice);
		// every side has at least two, since the cut-off is at most L/2
		const int lx = a.nc[0] >= 3 ? -1 : 0, hx = a.nc[0] >= 2 ? 1 : 0;
		const int ly = a.nc[1] >= 3 ? -1 : 0, hy = a.nc[1] >= 2 ? 1 : 0;
		const int lz = a.nc[2] >= 3 ? -1 : 0, hz = a.nc[2] >= 2 ? 1 : 0;
		for (int oz = lz; oz <= hz; oz++)
			for (int oy = ly; oy <= hy; oy++)
				for (int ox = lx; ox <= hx; ox++) {
					const int xx = (cx + ox + a.nc[0]) % a.nc[0];
					const int yy = (cy + oy + a.nc[1]) % a.nc[1];
					const int zz = (cz + oz + a.nc[2]) % a.nc[2];
					const int c = xx + a.nc[0] * (yy + a.nc[1] * zz);
					for (int j = sc->start[c], je = sc->start[c + 1]; j < je; j++) {
						if (j == s) continue;
						const int4 pj = sc->spos[j];
						const float dx = (float)(pi.x - pj.x) * a.fs[0];
						const float dy = (float)(pi.y - pj.y) * a.fs[1];
						const float dz = (float)(pi.z - pj.z) * a.fs[2];
						const float r2 = dx * dx + dy * dy + dz * dz;
						if (r2 >= a.rc2) continue;
						const float s2 = a.sig2 / r2, s6 = s2 * s2 * s2;
						const float ft = a.eps48 * s6 * (s6 - a.awh) * s2;
						e += a.eps4 * s6 * (s6 - a.aw) + a.ushift;
						fx += ft * dx; fy += ft * dy; fz += ft * dz;
					}
				}
		const int orig = pi.w;
		a.f[3 * orig] = fx;
		a.f[3 * orig + 1] = fy;
		a.f[3 * orig + 2] = fz;
	}
	// each pair is visited from both sides: half the energy per visit
	float v[1] = {0.5f * e};
	const int fld[1] = {0};
	block_to_slot<1>(v, fld, (long long *)&a.sc->esum, 0.f, -1);
}

__global__ void k_na_energy(const NaScratch *sc, double *epot)
{
	if (threadIdx.x == 0 && blockIdx.x == 0) *epot = (double)(long long)sc->esum * FX_ISCALE;
}

// the scratch array's device address on the current device (looked up once)
static int na_scratch(NaScratch **out)
{
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) { sepdev_set_error("cudaGetDevice", e); return SEPDEV_ECUDA; }
	if (dev < 0 || dev >= NA_MAXDEV) {
		sepdev_set_error("sep_gpu_lj_forces_noalloc: device index beyond the supported range",
				 cudaErrorInvalidDevice);
		return SEPDEV_EINVAL;
	}
	if (!g_na_addr[dev]) {
		void *p = NULL;
		e = cudaGetSymbolAddress(&p, g_na_scratch);
		if (e != cudaSuccess || !p) { sepdev_set_error("cudaGetSymbolAddress(scratch)", e); return SEPDEV_ECUDA; }
		g_na_addr[dev] = (NaScratch *)p;
	}
	*out = g_na_addr[dev];
	return SEPDEV_OK;
}

extern "C" int sep_gpu_lj_forces_noalloc(const double *x, long n, const double *L,
					 const double *param, double *f, double *epot, void *stream)
{
	if (n <= 0 || n > NA_MAXN) {
		sepdev_set_error("sep_gpu_lj_forces_noalloc: particle count outside 1..131072 "
				 "(the size of its fixed scratch array)", cudaErrorInvalidValue);
		return SEPDEV_EINVAL;
	}
	if (!L || !param || !(L[0] > 0) || !(L[1] > 0) || !(L[2] > 0) || !(param[0] > 0)) {
		sepdev_set_error("sep_gpu_lj_forces_noalloc: box lengths and cut-off must be positive",
				 cudaErrorInvalidValue);
		return SEPDEV_EINVAL;
	}
	if (2.0 * param[0] > L[0] || 2.0 * param[0] > L[1] || 2.0 * param[0] > L[2]) {
		sepdev_set_error("sep_gpu_lj_forces_noalloc: the cut-off exceeds half a box side",
				 cudaErrorInvalidValue);
		return SEPDEV_EINVAL;
	}
	int nc[3];
	long ncells = 1;
	for (int k = 0; k < 3; k++) {
		nc[k] = (int)floor(L[k] / param[0]);
		if (nc[k] < 1) nc[k] = 1;
		ncells *= nc[k];
	}
	if (ncells > NA_MAXC) {
		sepdev_set_error("sep_gpu_lj_forces_noalloc: more than 65536 linked cells "
				 "(box too large for the cut-off)", cudaErrorInvalidValue);
		return SEPDEV_EINVAL;
	}
	if (!x || !f || !epot) {
		sepdev_set_error("sep_gpu_lj_forces_noalloc: null device pointer", cudaErrorInvalidValue);
		return SEPDEV_EINVAL;
	}
	NaScratch *sc = NULL;
	int rc = na_scratch(&sc);
	if (rc) return rc;
	cudaStream_t st = (cudaStream_t)stream;
	const int ni = (int)n, B = 256;
	k_na_clear<<<(int)((ncells + B - 1) / B), B, 0, st>>>(sc, (int)ncells);
	k_na_bin<<<(ni + B - 1) / B, B, 0, st>>>(sc, x, ni, 1.0 / L[0], 1.0 / L[1], 1.0 / L[2],
						 nc[0], nc[1], nc[2]);
	k_na_scan<<<1, 1024, 0, st>>>(sc, (int)ncells);
	k_na_scatter<<<(ni + B - 1) / B, B, 0, st>>>(sc, ni);
	NaForceArgs a;
	a.sc = sc;
	a.n = ni;
	for (int k = 0; k < 3; k++) { a.nc[k] = nc[k]; a.fs[k] = (float)(L[k] / 4294967296.0); }
	const double cf = param[0], eps = param[1], sigma = param[2], aw = param[3];
	a.rc2 = (float)(cf * cf);
	a.sig2 = (float)(sigma * sigma);
	a.eps48 = (float)(48.0 * eps);
	a.eps4 = (float)(4.0 * eps);
	a.awh = (float)(0.5 * aw);
	a.aw = (float)aw;
	a.ushift = (float)(-4.0 * eps * (pow(sigma / cf, 12.) - aw * pow(sigma / cf, 6.)));
	a.f = f;
	k_na_force<<<(ni + B - 1) / B, B, 0, st>>>(a);
	k_na_energy<<<1, 32, 0, st>>>(sc, epot);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) { sepdev_set_error("sep_gpu_lj_forces_noalloc launch", e); return SEPDEV_ECUDA; }
	return SEPDEV_OK;
}
