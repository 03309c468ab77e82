// scan.cuh — deterministic three-phase inclusive scan over a generated
// sequence: tile sums -> one-block exclusive scan of the tile sums -> tile
// rescan with the carried prefix. Item i of tile t is summed in a fixed order
// (16 consecutive items per thread, then a block scan of the thread sums), so
// floating-point results depend only on n. A = double or unsigned long long.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace issm {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int64_t kScanTile = (int64_t)kScanThreads * kScanItems;

template <typename A> __device__ A block_exclusive_scan(A v, A *total) {
    __shared__ A warp_sums[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    A inc = v;
    for (int off = 1; off < 32; off <<= 1) {
        A o = __shfl_up_sync(0xffffffffu, inc, off);
        if (lane >= off) inc += o;
    }
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        A w = lane < nw ? warp_sums[lane] : A(0);
        for (int off = 1; off < 32; off <<= 1) {
            A o = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += o;
        }
        if (lane < nw) warp_sums[lane] = w;
    }
    __syncthreads();
    A warp_prefix = warp > 0 ? warp_sums[warp - 1] : A(0);
    *total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_prefix + inc - v;
}

template <typename A, typename Load>
__global__ void __launch_bounds__(kScanThreads) scan_tile_sums(int64_t n, Load load, A *tile_sums) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    A acc = A(0);
#pragma unroll
    for (int j = 0; j < kScanItems; ++j)
        if (base + j < n) acc += load(base + j);
    A total;
    block_exclusive_scan<A>(acc, &total);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// One block: exclusive scan of tile sums in place; tile_sums[tiles] = grand total.
template <typename A>
__global__ void __launch_bounds__(1024) scan_tile_prefix(A *tile_sums, int64_t tiles) {
    const int64_t per = (tiles + blockDim.x - 1) / blockDim.x;
    const int64_t lo = (int64_t)threadIdx.x * per;
    A acc = A(0);
    for (int64_t t = lo; t < lo + per && t < tiles; ++t) acc += tile_sums[t];
    A total;
    A prefix = block_exclusive_scan<A>(acc, &total);
    for (int64_t t = lo; t < lo + per && t < tiles; ++t) {
        A v = tile_sums[t];
        tile_sums[t] = prefix;
        prefix += v;
    }
    if (threadIdx.x == 0) tile_sums[tiles] = total;
}

template <typename A, typename Load, typename Write>
__global__ void __launch_bounds__(kScanThreads) scan_tile_apply(int64_t n, Load load, Write write,
                                                                const A *tile_sums, int64_t tiles) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    A items[kScanItems];
    A acc = A(0);
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        items[j] = (base + j < n) ? load(base + j) : A(0);
        acc += items[j];
    }
    A block_total;
    A prefix = block_exclusive_scan<A>(acc, &block_total) + tile_sums[blockIdx.x];
    const A grand = tile_sums[tiles];
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        prefix += items[j];
        if (base + j < n) write(base + j, prefix, grand);
    }
}

template <typename A, typename Load, typename Write>
int scan_apply(int64_t n, Load load, Write write, A *ws, cudaStream_t stream) {
    if (n <= 0) return 0;
    const int64_t tiles = (n + kScanTile - 1) / kScanTile;
    { scan_tile_sums<A, Load><<<(unsigned)tiles, kScanThreads, 0, stream>>>(n, load, ws); note_launch(); }
    { scan_tile_prefix<A><<<1, 1024, 0, stream>>>(ws, tiles); note_launch(); }
    { scan_tile_apply<A, Load, Write><<<(unsigned)tiles, kScanThreads, 0, stream>>>(n, load, write, ws, tiles); note_launch(); }
    return (int)cudaGetLastError();
}

}  // namespace issm
