// Stable LSD radix sort of (key, id) pairs, 8 bits per pass: per-block digit histograms, one scan
// over (digit, block) in digit-major order, and a scatter that keeps each block's items in input
// order (ranks within a warp from __match_any_sync, across warps from per-warp digit counts).
// Used by the deterministic adjoint of the differentiable renderer and by the alpha filter, which
// needs every tile's list in submission order.
#include <cuda_runtime.h>
#include <stdint.h>

#include "dsrg_kernels.h"

namespace dsrg {

namespace {

const int SORT_TILE = 4096;   // items per block
const int SORT_THREADS = 256;

__global__ void __launch_bounds__(SORT_THREADS) radix_histogram_kernel(const uint32_t *__restrict__ keys, uint64_t n, int shift,
                                                                       uint32_t *hist, uint32_t blocks) {
	__shared__ uint32_t counts[256];
	counts[threadIdx.x] = 0u;
	__syncthreads();
	const uint64_t begin = (uint64_t)blockIdx.x * SORT_TILE;
	for (int j = threadIdx.x; j < SORT_TILE; j += SORT_THREADS) {
		const uint64_t i = begin + j;
		if (i < n) atomicAdd(&counts[(keys[i] >> shift) & 0xFFu], 1u);
	}
	__syncthreads();
	hist[(size_t)threadIdx.x * blocks + blockIdx.x] = counts[threadIdx.x]; // digit-major
}

// Writes the block's items to their digit's slots in input order: 256 items at a time, ranks
// within a warp from __match_any_sync, across warps from per-warp digit counts, across steps
// from running per-digit counts.
__global__ void __launch_bounds__(SORT_THREADS) radix_scatter_kernel(const uint32_t *__restrict__ keysIn, const uint32_t *__restrict__ idsIn,
                                                                     uint64_t n, int shift, const uint32_t *__restrict__ offsets,
                                                                     uint32_t blocks, uint32_t *keysOut, uint32_t *idsOut) {
	__shared__ uint32_t running[256];
	__shared__ uint32_t warpCounts[SORT_THREADS / 32][256];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	running[threadIdx.x] = offsets[(size_t)threadIdx.x * blocks + blockIdx.x];
	for (int w = 0; w < SORT_THREADS / 32; w++) warpCounts[w][threadIdx.x] = 0u;
	__syncthreads();
	const uint64_t begin = (uint64_t)blockIdx.x * SORT_TILE;
	for (int j0 = 0; j0 < SORT_TILE; j0 += SORT_THREADS) {
		const uint64_t i = begin + j0 + threadIdx.x;
		const bool valid = i < n;
		const uint32_t key = valid ? keysIn[i] : 0u;
		const uint32_t digit = valid ? (key >> shift) & 0xFFu : 0x100u; // invalid lanes form their own group
		const uint32_t peers = __match_any_sync(0xFFFFFFFFu, digit);
		const uint32_t rankInWarp = __popc(peers & ((1u << lane) - 1u));
		if (valid && rankInWarp == 0) warpCounts[warp][digit] = __popc(peers);
		__syncthreads();
		if (valid) {
			uint32_t before = running[digit] + rankInWarp;
			for (int w = 0; w < warp; w++) before += warpCounts[w][digit];
			keysOut[before] = key;
			idsOut[before] = idsIn ? idsIn[i] : (uint32_t)i;
		}
		__syncthreads();
		uint32_t add = 0;
		for (int w = 0; w < SORT_THREADS / 32; w++) {
			add += warpCounts[w][threadIdx.x];
			warpCounts[w][threadIdx.x] = 0u;
		}
		running[threadIdx.x] += add;
		__syncthreads();
	}
}


} // namespace

uint32_t sort_blocks(uint64_t n) { return (uint32_t)((n + SORT_TILE - 1) / SORT_TILE); }

void launch_stable_sort(const uint32_t *keys, const uint32_t *ids, uint64_t n, int keyBits, const SortBuffers &b,
                        cudaStream_t stream, const uint32_t **sortedKeys, const uint32_t **sortedIds) {
	const uint32_t *kin = keys, *iin = ids;
	if (n > 0) {
		const uint32_t blocks = sort_blocks(n);
		const int passes = keyBits < 1 ? 1 : (keyBits + 7) / 8;
		uint32_t *kout = b.keysA, *iout = b.idsA;
		for (int p = 0; p < passes; p++) {
			const int shift = 8 * p;
			radix_histogram_kernel<<<blocks, SORT_THREADS, 0, stream>>>(kin, n, shift, b.hist, blocks);
			launch_scan(b.hist, b.offsets, 256u * blocks, b.scanScratch, b.scanScratchElems, stream);
			radix_scatter_kernel<<<blocks, SORT_THREADS, 0, stream>>>(kin, iin, n, shift, b.offsets, blocks, kout, iout);
			add_launches(2);
			kin = kout;
			iin = iout;
			kout = (kout == b.keysA) ? b.keysB : b.keysA;
			iout = (iout == b.idsA) ? b.idsB : b.idsA;
		}
	}
	*sortedKeys = kin;
	*sortedIds = iin;
}

} // namespace dsrg
