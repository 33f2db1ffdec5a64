// dev_cellsort.cuh - deterministic order inside a cell: members ranked by
// their x position (the high fixed-point word), ties by user index (shared
// by the single-system and batched pipelines).  Cells are rows along x, so
// this order makes a run of consecutive particles a compact slab along x,
// which shrinks the bounding box the list build stages candidates for.
#pragma once
#include "dev_common.cuh"

#define CS_MAX 384     // members a warp ranks in shared memory

__device__ __forceinline__ unsigned long long cs_key(const int *__restrict__ gid, const int4 *__restrict__ pos,
						      int v)
{
	return ((unsigned long long)(unsigned)pos[v].x << 32) | (unsigned)gid[v];
}

// One warp orders perm[lo, lo + cnt) by the key of perm[.].  Up to 32
// members are ranked in registers with shuffles, up to CS_MAX in the warp's
// shared arrays sk/sv (all lanes read the same key at a time: broadcasts),
// larger cells fall back to an insertion sort in lane 0.  Keys are
// distinct (user indices are), so every branch gives the same order.
__device__ __forceinline__ void cell_sort_warp(int lo, int cnt, const int *__restrict__ gid,
					       const int4 *__restrict__ pos, int *__restrict__ perm,
					       unsigned long long *sk, int *sv)
{
	const int lane = threadIdx.x & 31;
	if (cnt <= 1) return;
	if (cnt <= 32) {
		const int v = lane < cnt ? perm[lo + lane] : 0;
		const unsigned long long key = lane < cnt ? cs_key(gid, pos, v) : ~0ull;
		int rank = 0;
		for (int l = 0; l < cnt; l++) rank += (__shfl_sync(0xffffffffu, key, l) < key);
		__syncwarp();
		if (lane < cnt) perm[lo + rank] = v;
	} else if (cnt <= CS_MAX) {
		for (int e = lane; e < cnt; e += 32) {
			const int v = perm[lo + e];
			sv[e] = v;
			sk[e] = cs_key(gid, pos, v);
		}
		__syncwarp();
		for (int e0 = 0; e0 < cnt; e0 += 32) {
			const int e = e0 + lane;
			const unsigned long long key = e < cnt ? sk[e] : ~0ull;
			int rank = 0;
			for (int k = 0; k < cnt; k++) rank += (sk[k] < key);
			if (e < cnt) perm[lo + rank] = sv[e];
		}
		__syncwarp();
	} else if (lane == 0) {
		for (int x = lo + 1; x < lo + cnt; x++) {
			const int v = perm[x];
			const unsigned long long key = cs_key(gid, pos, v);
			int b = x - 1;
			while (b >= lo && cs_key(gid, pos, perm[b]) > key) { perm[b + 1] = perm[b]; b--; }
			perm[b + 1] = v;
		}
	}
}
