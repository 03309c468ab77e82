// moments_tc.cu — tensor-core form of the weighted moments that drive AMIS /
// N-PMC adaptation (_weighted_moments!, src/adaptive_gaussian_execution.jl:268-273).
//
// One streaming pass over the retained samples. For a tile of 128 samples,
// v = sqrt(w) (x - c) (c = previous proposal mean) is split v = vh + vl into
// bf16 parts, and so is sqrt(w) = sh + sl. One MMA per 16-sample K slice
// accumulates, in tensor memory, D = A B^T with A = [vh; vl] (M = 128 rows:
// 64 hi, 64 lo) and B = [vh; vl; sh; sl] (N = 144): all four hi/lo blocks of
// (vh + vl)(vh + vl)^T and the products with sh, sl. The epilogue adds them:
// S2 = sum w z z^T, S1 = sum w z of the split operand, and the converters sum
// S0 = sum (sh + sl)^2 the same way, so [S2 S1; S1^T S0] is the Gram matrix
// of the split operand (about 16 significant bits per element): the
// covariance, its Schur complement, is positive semidefinite up to FP32
// accumulation however few samples carry the weight, and the regularising
// ridge keeps the fit positive definite. Each CTA stores P = S / 2; the
// reduce kernel forms S = P + P^T.
//
// When the new mean lies far from c relative to the spread, S2/S0 and the
// mean's outer product nearly cancel. A second pass centred at the first
// pass's mean runs when the first pass's cancellation error could matter
// against the variance or the fit's ridge (see the reduce kernel); its
// kernels are always launched (graph replays see a fixed sequence) and
// return at once when the flag is clear.
//
// A is stored MN-major: each sample's 8-coordinate groups are 16-byte chunks,
// so four threads convert a sample row straight from the staged tile. Warp
// roles: warp 0 issues the MMAs; warps 1..16 build the operand (three
// buffers, so conversion runs up to two tiles ahead of the MMAs) from the
// staged tiles; warp 17 stages the tiles. For d = 32 or 64 (aligned arrays)
// the stager keeps a three-deep ring of stages filled by tensor copies
// (cp.async.bulk.tensor through a tensor map of the samples: one or two
// 32-float x 128-row boxes per tile, 128-byte swizzle, so converters read
// rows without bank conflicts, plus one bulk copy of the tile's log weights;
// completion counted in bytes on the stage's mbarrier); converters wait on
// that mbarrier and release the stage with one arrival per warp, so no role
// ever waits on a CTA-wide barrier. Other shapes stage padded rows with
// cp.async from the converters. Per-CTA partials are summed across CTAs
// (compensated FP32) and mean = c + S1/S0, cov = S2/S0 - (S1/S0)(S1/S0)^T in
// FP64.
#include <cstring>

#include "issm_device.cuh"
#include "issm_internal.h"
#include "tcgen05.cuh"

namespace issm {

// 16 converter warps (four threads per sample row, two coordinate groups
// each): the conversion is latency-bound, and with one CTA per SM (shared
// memory) only more warps hide its dependency chains
constexpr int kMtConvWarps = 16;
constexpr int kMtConvThreads = 32 * kMtConvWarps;
constexpr int kMtStagerWarp = 1 + kMtConvWarps;
constexpr int kMtThreads = 32 * (2 + kMtConvWarps);  // issuer, converters, stager
constexpr int kMtTile = 128;   // samples per tile = MMA K extent per tile
constexpr int kMtTPR = kMtConvThreads / kMtTile;  // converter threads per sample row
constexpr int kMtGPT = 8 / kMtTPR;                // coordinate groups (of 8) per converter thread
constexpr int kMtCtasPerSm = 1;  // CTAs per SM (two 64-sample pipelines measured the same)
constexpr int kMtCols = 80;    // columns of a CTA's partial (64 coordinates, sqrt(w), padding)
constexpr int kMtN = 144;      // MMA N: hi rows, lo rows, sqrt(w) hi and lo, padding
constexpr int kMtStages = 3;   // staged sample tiles in flight
constexpr int kMtABufs = 3;    // operand buffers: conversion runs up to two tiles ahead of the MMAs
constexpr int kMtRS = 68;      // padded row of a staged tile (floats): conflict-free row reads
constexpr int kMtWOff = kMtTile * kMtRS * 4;  // byte offset of the tile's log weights in a stage
// rows (padded, or two swizzled boxes), then the log weights; a 1024-byte multiple
constexpr int kMtRawBytes = (kMtWOff + kMtTile * 4 + 1023) / 1024 * 1024;
// One operand buffer holds 18 row groups of 128 samples x 16 bytes, MN-major:
// groups 0..7 the bf16 hi parts of the 64 coordinates, groups 8..15 their lo
// parts, group 16 (sqrt(w) hi, sqrt(w) lo, zeros) and group 17 zeros. A is
// its first 16 groups (M = 128), B all 18 (N = 144).
constexpr int kMtGroups = 18;
constexpr int kMtBuf = kMtGroups * kMtTile * 16;
// operand buffers, stages (1024-byte multiples: the swizzled boxes need 1024-byte
// aligned destinations), centre; plus 1024 bytes to align the base
constexpr size_t kMtSmem = (size_t)kMtABufs * kMtBuf + (size_t)kMtStages * kMtRawBytes + 256 + 1024;
static_assert(kMtSmem <= 232448 - 2048, "dynamic shared memory per CTA");
static_assert(kMtBuf % 1024 == 0 && kMtRawBytes % 1024 == 0, "stages start on 1024-byte boundaries");
static_assert(128 * 65 * 4 <= kMtRawBytes, "the epilogue's row sums fit in one stage");
constexpr int kMtPartial = 65 * kMtCols;  // P = S / 2 of one CTA (the reduce forms S = P + P^T)

__global__ void __launch_bounds__(kMtThreads, kMtCtasPerSm) moments_tc_kernel(const float *__restrict__ x, int d, int64_t n,
                                                                    const float *__restrict__ lw,
                                                                    const double *__restrict__ summary,
                                                                    const double *__restrict__ center,
                                                                    float *__restrict__ partial, int *error,
                                                                    const int *__restrict__ gate,
                                                                    const __grid_constant__ CUtensorMap tmap,
                                                                    int tma) {
    if (gate != nullptr && *gate == 0) return;  // refinement pass not needed
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // the swizzled boxes need 1024-byte aligned stages
    unsigned char *smem = smem_raw + ((1024 - (tc::smem_u32(smem_raw) & 1023)) & 1023);
    unsigned char *s_a = smem;                                    // [buf] x kMtBuf
    unsigned char *s_raw = smem + (size_t)kMtABufs * kMtBuf;
    float *s_c = reinterpret_cast<float *>(s_raw + (size_t)kMtStages * kMtRawBytes);
    __shared__ __align__(8) uint64_t a_full[kMtABufs], a_empty[kMtABufs], raw_full[kMtStages], raw_empty[kMtStages];
    __shared__ uint32_t tmem_base;
    __shared__ volatile int abort_flag;
    __shared__ float s_s0[kMtConvWarps];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) tc::tmem_alloc(&tmem_base, 256);
    if (tid == 0) {
        for (int b = 0; b < kMtABufs; ++b) {
            tc::mbar_init(&a_full[b], kMtConvWarps);
            tc::mbar_init(&a_empty[b], 1);
        }
        for (int s = 0; s < kMtStages; ++s) {
            tc::mbar_init(&raw_full[s], 1);
            tc::mbar_init(&raw_empty[s], kMtConvWarps);
        }
        tc::fence_mbar_init();
        abort_flag = 0;
    }
    for (int c = tid; c < 64; c += kMtThreads) s_c[c] = c < d ? (float)center[c] : 0.f;
    // group 17 of every buffer: zeros (B rows 136..143, never read back)
    for (int e = tid; e < kMtABufs * kMtTile; e += kMtThreads)
        *reinterpret_cast<uint4 *>(s_a + (size_t)(e / kMtTile) * kMtBuf + 17 * kMtTile * 16 + (e % kMtTile) * 16) =
            make_uint4(0u, 0u, 0u, 0u);
    if (tid < kMtConvWarps) s_s0[tid] = 0.f;
    const float m = (float)summary[0];
    const float inv_sqrt_s = (float)(1.0 / sqrt(summary[1]));
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tmem_base;  // D: 128 lanes x 144 columns
    const int64_t ntiles = (n + kMtTile - 1) / kMtTile;
    const int my_tiles = (int)((ntiles - (int64_t)blockIdx.x + gridDim.x - 1) / gridDim.x);
    auto tile_of = [&](int it) -> int64_t { return (int64_t)blockIdx.x + (int64_t)it * gridDim.x; };
    auto tile_rows = [&](int it) -> int { return (int)min((int64_t)kMtTile, n - tile_of(it) * kMtTile); };
    auto wait = [&](uint64_t *bar, uint32_t parity) -> bool {
        if (abort_flag) return false;
        if (tc::mbar_wait(bar, parity)) return true;
        atomicExch(error, 1);
        abort_flag = 1;
        return false;
    };
    // tensor copies of the tiles (d = 32 or 64, aligned arrays; the host
    // encoded the tensor map); else padded rows by cp.async
    const bool bulk = tma != 0;
    const int nbox = d > 32 ? 2 : 1;

    if (warp == 0) {
        // ---- issuer: D += [Ah; Al] [Ah; Al; sqrt(w)]^T, one MMA per K slice ----
        const uint32_t idesc = tc::instr_desc(tc::kBF16, 128, kMtN) | tc::kMajorMN;
        constexpr uint32_t LBO = 128, SBO = kMtTile * 16;  // K-group stride, row-group stride
        for (int it = 0; it < my_tiles; ++it) {
            const int buf = it % kMtABufs;
            if (lane == 0) {
                const bool ok = wait(&a_full[buf], (uint32_t)((it / kMtABufs) & 1));
                tc::fence_after_sync();
                if (ok) {
                    const uint32_t a0 = tc::smem_u32(s_a + (size_t)buf * kMtBuf);
#pragma unroll
                    for (int s = 0; s < kMtTile / 16; ++s) {
                        const uint64_t da = tc::smem_desc(a0 + s * 256, LBO, SBO);
                        tc::mma(tbase, da, da, idesc, it > 0 || s > 0);
                    }
                }
                tc::commit(&a_empty[buf]);
            }
            __syncwarp();
        }
    } else if (warp == kMtStagerWarp) {
        // ---- stager: the tile's one or two swizzled boxes by tensor copies,
        // its log weights (whole 16-byte groups) by one bulk copy ----
        if (bulk) {
            int issued = 0;
            for (int it = 0; it < my_tiles; ++it) {
                const int s = it % kMtStages;
                if (it >= kMtStages) {
                    int ok = 1;
                    if (lane == 0) ok = wait(&raw_empty[s], (uint32_t)(((it / kMtStages) - 1) & 1));
                    if (!__shfl_sync(0xffffffffu, ok, 0)) break;
                }
                const int64_t row0 = tile_of(it) * kMtTile;
                const int rows = tile_rows(it);
                const uint32_t wb = (uint32_t)(rows & ~3) * 4u;
                unsigned char *dst = s_raw + (size_t)s * kMtRawBytes;
                if (lane == 0) {
                    // a box counts all its bytes (rows past n arrive as zeros)
                    tc::mbar_arrive_expect_tx(&raw_full[s], (uint32_t)nbox * 16384u + wb);
                    for (int b = 0; b < nbox; ++b)
                        tc::tma_load_2d(dst + (size_t)b * 16384, &tmap, 32 * b, (int)row0, &raw_full[s]);
                    if (wb > 0) tc::bulk_copy_g2s(dst + kMtWOff, lw + row0, wb, &raw_full[s]);
                }
                __syncwarp();
                issued = it + 1;
            }
            // every copy lands before the CTA can exit (the converters consume
            // them all unless a wait timed out)
            if (lane == 0)
                for (int it = max(0, issued - kMtStages); it < issued; ++it)
                    tc::mbar_wait(&raw_full[it % kMtStages], (uint32_t)((it / kMtStages) & 1));
        }
    } else {
        // ---- converters: build [Ah; Al; sqrt(w)] from the staged tiles ----
        const int ctid = tid - 32;
        auto issue_raw = [&](int it) {  // cp.async staging (shapes without tensor copies)
            if (it < my_tiles) {
                const int64_t row0 = tile_of(it) * kMtTile;
                const int rows = tile_rows(it);
                float *dst = reinterpret_cast<float *>(s_raw + (size_t)(it % kMtStages) * kMtRawBytes);
                float *dlw = dst + kMtTile * kMtRS;
                const float *src = x + row0 * d;
                const bool vec = (d % 4 == 0) && ((reinterpret_cast<uintptr_t>(x) & 15) == 0);
                if (vec) {
                    const int q4 = d >> 2, total = rows * q4;
                    for (int e = ctid; e < total; e += kMtConvThreads) {
                        const int r = e / q4, c4 = e - r * q4;
                        tc::cp_async16(dst + r * kMtRS + c4 * 4, src + (size_t)r * d + c4 * 4);
                    }
                } else {
                    for (int e = ctid; e < rows * d; e += kMtConvThreads) {
                        const int r = e / d, c = e - r * d;
                        tc::cp_async4(dst + r * kMtRS + c, src + (size_t)r * d + c);
                    }
                }
                for (int r = ctid; r < rows; r += kMtConvThreads) tc::cp_async4(dlw + r, lw + row0 + r);
            }
            tc::cp_async_commit();
        };
        if (!bulk)
            for (int s = 0; s < kMtStages; ++s) issue_raw(s);
        const int k = ctid % kMtTile, part = ctid / kMtTile;
        float s0 = 0.f;  // sum of (sqrt(w) hi + lo)^2 over this thread's samples: S0 of the split operand
        for (int it = 0; it < my_tiles; ++it) {
            const int buf = it % kMtABufs, stage = it % kMtStages;
            bool ok = true;
            if (bulk) {
                // every lane acquires the stage's bytes itself; the outcome is made warp-uniform
                ok = __all_sync(0xffffffffu, wait(&raw_full[stage], (uint32_t)((it / kMtStages) & 1)));
            } else {
                tc::cp_async_wait<kMtStages - 1>();
                tc::named_sync(1, kMtConvThreads);
            }
            if (it >= kMtABufs && ok) {
                if (lane == 0) ok = wait(&a_empty[buf], (uint32_t)(((it / kMtABufs) - 1) & 1));
                ok = __shfl_sync(0xffffffffu, (int)ok, 0) != 0;
            }
            if (ok) {
                const unsigned char *stage_p = s_raw + (size_t)stage * kMtRawBytes;
                const float *raw = reinterpret_cast<const float *>(stage_p);
                // coordinates c .. c + 3 of this thread's row: swizzled box or padded row
                auto row_at = [&](int c) -> const float4 * {
                    return reinterpret_cast<const float4 *>(bulk ? tc::swizzled_row_chunk(stage_p, k, c)
                                                                 : raw + k * kMtRS + c);
                };
                unsigned char *ab = s_a + (size_t)buf * kMtBuf;
                const int64_t i = tile_of(it) * kMtTile + k;
                const bool active = i < n;
                // the bulk copy carries whole 16-byte groups of weights; the
                // (at most three) beyond them come from global memory
                const int staged_w = bulk ? (tile_rows(it) & ~3) : kMtTile;
                const float l = !active ? -INFINITY : (k < staged_w ? raw[kMtWOff / 4 + k] : lw[i]);
                const float sw = l == -INFINITY ? 0.f : expf(0.5f * (l - m)) * inv_sqrt_s;
                const bool full = active && d == 64;
#pragma unroll
                for (int gg = 0; gg < kMtGPT; ++gg) {
                    const int g = part * kMtGPT + gg, c = g * 8;
                    float v[8];
                    const float4 c0 = *reinterpret_cast<const float4 *>(s_c + c),
                                 c1 = *reinterpret_cast<const float4 *>(s_c + c + 4);
                    if (full) {
                        const float4 f0 = *row_at(c);
                        const float4 f1 = *row_at(c + 4);
                        v[0] = sw * (f0.x - c0.x);
                        v[1] = sw * (f0.y - c0.y);
                        v[2] = sw * (f0.z - c0.z);
                        v[3] = sw * (f0.w - c0.w);
                        v[4] = sw * (f1.x - c1.x);
                        v[5] = sw * (f1.y - c1.y);
                        v[6] = sw * (f1.z - c1.z);
                        v[7] = sw * (f1.w - c1.w);
                    } else {
                        float4 f0 = make_float4(0.f, 0.f, 0.f, 0.f), f1 = f0;
                        if (active) {
                            f0 = *row_at(c);
                            f1 = *row_at(c + 4);
                        }
                        v[0] = (active && c < d) ? sw * (f0.x - c0.x) : 0.f;
                        v[1] = (active && c + 1 < d) ? sw * (f0.y - c0.y) : 0.f;
                        v[2] = (active && c + 2 < d) ? sw * (f0.z - c0.z) : 0.f;
                        v[3] = (active && c + 3 < d) ? sw * (f0.w - c0.w) : 0.f;
                        v[4] = (active && c + 4 < d) ? sw * (f1.x - c1.x) : 0.f;
                        v[5] = (active && c + 5 < d) ? sw * (f1.y - c1.y) : 0.f;
                        v[6] = (active && c + 6 < d) ? sw * (f1.z - c1.z) : 0.f;
                        v[7] = (active && c + 7 < d) ? sw * (f1.w - c1.w) : 0.f;
                    }
                    const uint4 hi = make_uint4(tc::pack_bf16x2(v[0], v[1]), tc::pack_bf16x2(v[2], v[3]),
                                                tc::pack_bf16x2(v[4], v[5]), tc::pack_bf16x2(v[6], v[7]));
                    auto lo2 = [](float a, float b, uint32_t h) {
                        return tc::pack_bf16x2(a - __uint_as_float(h << 16), b - __uint_as_float(h & 0xffff0000u));
                    };
                    const uint4 lo = make_uint4(lo2(v[0], v[1], hi.x), lo2(v[2], v[3], hi.y), lo2(v[4], v[5], hi.z),
                                                lo2(v[6], v[7], hi.w));
                    *reinterpret_cast<uint4 *>(ab + (size_t)g * kMtTile * 16 + k * 16) = hi;
                    *reinterpret_cast<uint4 *>(ab + (size_t)(8 + g) * kMtTile * 16 + k * 16) = lo;
                }
                if (part == kMtTPR - 1) {
                    // group 16: sqrt(w) hi in row 128, its lo part in row 129
                    const uint32_t h = tc::pack_bf16x2(sw, 0.f);
                    const float swh = __uint_as_float(h << 16);
                    const uint32_t hl = tc::pack_bf16x2(swh, sw - swh);
                    const float swl = __uint_as_float(hl & 0xffff0000u);
                    const float sws = swh + swl;  // exact: swl is a bf16 below swh's last bit
                    s0 = fmaf(sws, sws, s0);
                    *reinterpret_cast<uint4 *>(ab + (size_t)16 * kMtTile * 16 + k * 16) = make_uint4(hl, 0u, 0u, 0u);
                }
            }
            tc::fence_proxy_async();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&a_full[buf]);
            if (bulk) {
                if (lane == 0) tc::mbar_arrive(&raw_empty[stage]);  // this warp is done with the stage
            } else {
                tc::named_sync(1, kMtConvThreads);  // the stage is consumed: refill it
                issue_raw(it + kMtStages);
            }
        }
        if (!bulk) tc::cp_async_wait_all();
        // S0 per warp in a fixed order (lanes by xor tree, warps summed in order below)
        for (int off = 16; off > 0; off >>= 1) s0 += __shfl_xor_sync(0xffffffffu, s0, off);
        if (lane == 0) s_s0[warp - 1] = s0;
    }
    // ---- the last commit tracks every MMA of the CTA ----
    tc::fence_before_sync();
    __syncthreads();
    if (my_tiles > 0) {
        const int last = my_tiles - 1;
        if (!tc::mbar_wait(&a_empty[last % kMtABufs], (uint32_t)((last / kMtABufs) & 1)) && tid == 0) {
            atomicExch(error, 1);
            abort_flag = 1;
        }
    }
    __syncthreads();
    tc::fence_after_sync();
    float *out = partial + (size_t)blockIdx.x * kMtPartial;
    // row sums T[r][j] = D[r][j] + D[r][64 + j] (j < 64) and T[r][64] =
    // D[r][128] + D[r][129] in the first stage's space (every copy has landed)
    float *T = reinterpret_cast<float *>(s_raw);
    // warps 1..4 read TMEM lane quadrants 1, 2, 3, 0 (a warp reads quadrant warp % 4)
    if (!abort_flag && warp >= 1 && warp <= 4) {
        const int q = warp & 3, row = 32 * q + lane;
        const uint32_t lane_base = tbase + ((uint32_t)(32 * q) << 16);
#pragma unroll
        for (int c0 = 0; c0 < 64; c0 += 16) {
            float a[16], b[16];
            if (my_tiles > 0) {
                tc::tmem_ld16(lane_base + (uint32_t)c0, a);
                tc::tmem_ld16(lane_base + (uint32_t)(64 + c0), b);
            } else {
                for (int j = 0; j < 16; ++j) a[j] = b[j] = 0.f;
            }
            for (int j = 0; j < 16; ++j) T[row * 65 + c0 + j] = a[j] + b[j];
        }
        float a[16];
        if (my_tiles > 0) tc::tmem_ld16(lane_base + 128u, a);
        else for (int j = 0; j < 16; ++j) a[j] = 0.f;
        T[row * 65 + 64] = a[0] + a[1];
    }
    __syncthreads();
    // P = S / 2 over 65 x 80: S2 = T[i] + T[64 + i], S1 the sqrt(w) column, S0 from the converters
    if (!abort_flag) {
        float s0_all = 0.f;
        for (int w = 0; w < kMtConvWarps; ++w) s0_all += s_s0[w];
        for (int e = tid; e < kMtPartial; e += kMtThreads) {
            const int r = e / kMtCols, c = e - r * kMtCols;
            float v = 0.f;
            if (r < 64 && c < 65) v = T[r * 65 + c] + T[(64 + r) * 65 + c];
            else if (r == 64 && c < 64) v = T[c * 65 + 64] + T[(64 + c) * 65 + 64];
            else if (r == 64 && c == 64) v = s0_all;
            out[e] = 0.5f * v;
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 256);
}

// Partials are [block][65][80] FP32 (P = S / 2). Every CTA sums 32 entries
// over the blocks (32 block-strided lanes per entry, coalesced); the last CTA
// to finish (a device-scope counter, reset by that CTA) forms S = P + P^T and
// from it mean = c + S1/S0 and cov = S2/S0 - (S1/S0)(S1/S0)^T in FP64, with c
// the FP32 value the pass subtracted. `center` and `mean` may be the same
// array: each entry is read before it is written. With `refine` given, the
// last CTA sets it when, on some diagonal, the pass's cancellation error
// (2^-16 of the second moment s2 about c) exceeds 2^-8 of the variance v plus
// 2^-4 of R = sqrt(eps(Float32)) tr(L L^T) / d for the previous factor L, the
// scale of the ridge the fit adds (R = 0 without L): s2 > 256 v + 4096 R.
// Low-ESS rounds whose variance is mostly ridge then refine only when the
// mean moved by more than about one previous scale.
constexpr int kMtReduceThreads = 1024;  // 32 entries x 32 block-strided lanes per CTA

// FP64 work here runs on one SM's FP64 pipe (a warp-instruction holds it for
// about 64 cycles on this GPU whatever the active lanes), so the kernel keeps
// FP64 to the Schur complement itself: lanes combine in compensated FP32, the
// ridge scale is FP32, 1/S0 is formed once, and only the lower triangle of the
// covariance is computed (four FP64 operations per element).
__global__ void __launch_bounds__(kMtReduceThreads) moments_tc_reduce_kernel(
    const float *__restrict__ partial, int blocks, double *sums, int d, const double *center, double *mean,
    double *__restrict__ cov, const int *__restrict__ gate, int *refine, const float *__restrict__ prev,
    unsigned *counter) {
    if (gate != nullptr && *gate == 0) return;
    __shared__ float acc_s[32][33], cmp_s[32][33];
    __shared__ double s_m[65];  // S1 / S0 (the mean about c)
    __shared__ double s_inv;
    __shared__ float s_r[32];
    __shared__ int last;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int e = blockIdx.x * 32 + tx;
    // compensated FP32 over this lane's blocks, then over the 32 lanes
    float s = 0.f, cmp = 0.f;
    if (e < kMtPartial)
        for (int b = ty; b < blocks; b += 32) {
            const float y = partial[(size_t)b * kMtPartial + e] - cmp;
            const float t = s + y;
            cmp = (t - s) - y;
            s = t;
        }
    acc_s[ty][tx] = s;
    cmp_s[ty][tx] = cmp;
    __syncthreads();
    if (ty == 0 && e < kMtPartial) {
        float t = 0.f, c = 0.f;
        for (int r = 0; r < 32; ++r) {
            const float y = acc_s[r][tx] - (cmp_s[r][tx] + c);
            const float u = t + y;
            c = (u - t) - y;
            t = u;
        }
        sums[e] = (double)t - (double)c;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    auto S = [&](int r, int c) { return __ldcg(sums + r * kMtCols + c) + __ldcg(sums + c * kMtCols + r); };
    if (threadIdx.x == 0) s_inv = 1.0 / S(64, 64);
    // R = sqrt(eps(Float32)) tr(L L^T) / d of the previous factor (0 without one), in FP32
    float rr = 0.f;
    if (refine != nullptr && prev != nullptr)
        for (int q = threadIdx.x; q < d * d; q += blockDim.x) rr = fmaf(prev[q], prev[q], rr);
    for (int off = 16; off > 0; off >>= 1) rr += __shfl_xor_sync(0xffffffffu, rr, off);
    if (tx == 0) s_r[ty] = rr;
    __syncthreads();
    if (threadIdx.x < 65) s_m[threadIdx.x] = S(64, threadIdx.x) * s_inv;
    __syncthreads();
    const double inv = s_inv;
    // lower triangle, row-major: q -> (r, c), c <= r
    const int tri = d * (d + 1) / 2;
    for (int q = threadIdx.x; q < tri; q += blockDim.x) {
        int r = (int)((sqrtf(8.f * (float)q + 1.f) - 1.f) * 0.5f);
        if ((r + 1) * (r + 2) / 2 <= q) ++r;
        if (r * (r + 1) / 2 > q) --r;
        const int c = q - r * (r + 1) / 2;
        const double v = fma(S(r, c), inv, -s_m[r] * s_m[c]);
        cov[r + (size_t)c * d] = v;
        cov[c + (size_t)r * d] = v;
    }
    int flag = 0;
    if (refine != nullptr && threadIdx.x < d) {
        float ridge = 0.f;
        for (int w = 0; w < 32; ++w) ridge += s_r[w];
        ridge *= 3.4526698e-4f / (float)d;  // sqrt(FLT_EPSILON)
        const int r = threadIdx.x;
        const double s2 = S(r, r) * inv, v = s2 - s_m[r] * s_m[r];
        // the pass's error (2^-16 of s2) above 2^-8 of v plus 2^-4 of the ridge scale
        flag = !(s2 <= 256.0 * v + 4096.0 * (double)ridge);
    }
    flag = __syncthreads_or(flag);  // also orders the reads of `center` below after every thread's work above
    for (int j = threadIdx.x; j < d; j += blockDim.x) mean[j] = (double)(float)center[j] + s_m[j];
    if (threadIdx.x == 0) {
        if (refine != nullptr) *refine = flag;
        *counter = 0u;
    }
}

constexpr int kMtMaxBlocks = kSMs * kMtCtasPerSm;

static int moments_tc_blocks(int64_t n) {
    const int64_t t = (n + kMtTile - 1) / kMtTile;
    const int64_t cap = (int64_t)device_sms() * kMtCtasPerSm;  // <= kMtMaxBlocks, the scratch bound
    return (int)(t < cap ? (t < 1 ? 1 : t) : cap);
}

size_t moments_tc_workspace_bytes(int64_t n) {
    (void)n;
    return sizeof(float) * (size_t)kMtMaxBlocks * kMtPartial + sizeof(double) * kMtPartial + 256;
}

int moments_tc(const void *x, int d, int64_t n, const void *lw, const double *summary, const double *shift,
               const float *prev_factor, double *mean, double *cov, int precision, void *ws, size_t ws_bytes,
               int *error, cudaStream_t stream) {
    (void)precision;  // both tensor-core forms use the bf16 split contraction
    if (d > 64) return ISSM_E_UNSUPPORTED;
    if (ws_bytes < moments_tc_workspace_bytes(n)) return ISSM_E_WORKSPACE;
    const int blocks = moments_tc_blocks(n);
    float *partial = (float *)ws;
    const int e = allow_dynamic_smem((const void *)moments_tc_kernel);
    if (e) return e;
    double *sums = reinterpret_cast<double *>(partial + (size_t)kMtMaxBlocks * kMtPartial);
    int *refine = reinterpret_cast<int *>(sums + kMtPartial);
    unsigned *counter = reinterpret_cast<unsigned *>(error + 1);  // zero with the workspace; reset by each use
    const int rblocks = (kMtPartial + 31) / 32;
    // pass 1 about `shift`
    // tensor copies of the tiles when the shape allows (one map per call; both passes read it)
    CUtensorMap tmap;
    memset(&tmap, 0, sizeof(tmap));
    int tma = 0;
    if (row_tiles_supported(x, d, n) && ((reinterpret_cast<uintptr_t>(lw) & 15) == 0))
        tma = encode_row_tiles(&tmap, x, d, n) == ISSM_OK ? 1 : 0;
    { moments_tc_kernel<<<blocks, kMtThreads, kMtSmem, stream>>>((const float *)x, d, n, (const float *)lw,
                                                                       summary, shift, partial, error, nullptr,
                                                                       tmap, tma);
      note_launch(); }
    { moments_tc_reduce_kernel<<<rblocks, kMtReduceThreads, 0, stream>>>(partial, blocks, sums, d, shift, mean, cov,
                                                                         nullptr, refine, prev_factor, counter);
      note_launch(); }
    // pass 2 about the new mean (kernels return at once unless pass 1 set `refine`)
    { moments_tc_kernel<<<blocks, kMtThreads, kMtSmem, stream>>>((const float *)x, d, n, (const float *)lw,
                                                                      summary, mean, partial, error, refine, tmap,
                                                                      tma);
      note_launch(); }
    { moments_tc_reduce_kernel<<<rblocks, kMtReduceThreads, 0, stream>>>(partial, blocks, sums, d, mean, mean, cov,
                                                                         refine, nullptr, nullptr, counter);
      note_launch(); }
    return (int)cudaGetLastError();
}

}  // namespace issm
