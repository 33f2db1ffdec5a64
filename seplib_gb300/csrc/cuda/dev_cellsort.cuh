// dev_cellsort.cuh - deterministic order inside a cell: members ranked by
// their user index (shared by the single-system and batched pipelines).
#pragma once
#include "dev_common.cuh"

#define CS_MAX 512     // members a warp ranks in shared memory

// One warp orders perm[lo, lo + cnt) by gid[perm[.]].  Up to 32 members are
// ranked in registers with shuffles, up to CS_MAX in the warp's shared
// arrays sk/sv (all lanes read the same key at a time: broadcasts), larger
// cells fall back to an insertion sort in lane 0.  Keys are distinct, so
// every branch gives the same order.
__device__ __forceinline__ void cell_sort_warp(int lo, int cnt, const int *__restrict__ gid,
					       int *__restrict__ perm, int *sk, int *sv)
{
	const int lane = threadIdx.x & 31;
	if (cnt <= 1) return;
	if (cnt <= 32) {
		const int v = lane < cnt ? perm[lo + lane] : 0;
		const int key = lane < cnt ? gid[v] : 0x7fffffff;
		int rank = 0;
		for (int l = 0; l < cnt; l++) rank += (__shfl_sync(0xffffffffu, key, l) < key);
		__syncwarp();
		if (lane < cnt) perm[lo + rank] = v;
	} else if (cnt <= CS_MAX) {
		for (int e = lane; e < cnt; e += 32) {
			const int v = perm[lo + e];
			sv[e] = v;
			sk[e] = gid[v];
		}
		__syncwarp();
		for (int e0 = 0; e0 < cnt; e0 += 32) {
			const int e = e0 + lane;
			const int key = e < cnt ? sk[e] : 0x7fffffff;
			int rank = 0;
			for (int k = 0; k < cnt; k++) rank += (sk[k] < key);
			if (e < cnt) perm[lo + rank] = sv[e];
		}
		__syncwarp();
	} else if (lane == 0) {
		for (int x = lo + 1; x < lo + cnt; x++) {
			int v = perm[x], key = gid[v], b = x - 1;
			while (b >= lo && gid[perm[b]] > key) { perm[b + 1] = perm[b]; b--; }
			perm[b + 1] = v;
		}
	}
}
