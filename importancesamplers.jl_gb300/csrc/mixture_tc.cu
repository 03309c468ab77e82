// mixture_tc.cu — tensor-core (tcgen05) form of the factor-bank mixture
// density for FP32 samples: the Mahalanobis contraction runs as an MMA and
// the radial density plus the balance-heuristic log-sum-exp run in the
// epilogue straight out of tensor memory.
//
// For every component k the reference solves L_k z = x - mu_k by forward
// substitution (_packed_gaussian_logdensity!, src/native_execution.jl:346-384).
// Here W_k = L_k^-1 (FP32, cached per slot in issm_bank.inverse_factors) and
// the samples are centred on one shift c (the generating / appended slot's
// mean):
//   z_k = W_k (x - c) - b_k,   b_k = W_k (mu_k - c),
// so each 128-sample tile is one GEMM  D[128 x K*DP] = X'[128 x DP] W^T.
// Precision forms (FP32 accumulation in TMEM in both):
//   TF32    one kind::tf32 MMA per K slice, operands rounded to tf32 (RNE);
//   BF16x3  operands split v = hi + lo in bf16, D = Xh Wh + Xl Wh + Xh Wl,
//           about 16 significant bits per product.
//
// Two kernels per launch:
//   tc_prepare_kernel  one CTA per slot: W_k in MMA operand form (bf16 hi/lo
//                      or tf32, row-contiguous canonical layout) and b_k;
//   mixture_tc_kernel  persistent, 8 warps, one 128-sample tile at a time:
//     * sample tiles stream in with cp.async (16-byte, L1 bypass) into a ring
//       of padded shared-memory stages, prefetched raw_stages tiles ahead;
//     * all threads centre, round and split the tile into the A operand
//       (double-buffered, so converting tile t+1 overlaps MMAs of tile t);
//     * component operands arrive by bulk copies on an mbarrier, double-
//       buffered by chunk when a tile needs several chunks of components;
//     * one thread issues the MMAs of item j (tile, component chunk) into one
//       of two TMEM accumulators while all warps run the epilogue of item
//       j-1 from the other: warp w reads TMEM lanes 32 (w mod 4).. and takes
//       the components of parity w / 4; the two halves merge their
//       log-sum-exp states through shared memory when the tile completes.
// Every wait is bounded; a timeout sets the sticky error word and the CTA
// unwinds after draining its outstanding copies and MMAs.
#include "issm_device.cuh"
#include "issm_internal.h"
#include "tcgen05.cuh"
#include "trinv.cuh"

namespace issm {

constexpr int kTcTile = 128;
constexpr size_t kTcMaxSmem = 232448 - 1024;  // dynamic shared memory per CTA, static part reserved

__device__ __forceinline__ uint32_t tf32_bits(float f) {
    uint32_t u = __float_as_uint(f);
    if ((u & 0x7f800000u) == 0x7f800000u) return u;
    u += 0xFFFu + ((u >> 13) & 1u);
    return u & ~0x1FFFu;
}

// 16 bytes of operand values from v[PER]: 4 tf32 (nearest even), or 8 bf16
// (the hi part; pack_lo gives the lo part bf16(v - hi)).
template <int KIND> __device__ __forceinline__ uint4 pack_hi(const float *v) {
    if (KIND == tc::kTF32) return make_uint4(tc::tf32_rn(v[0]), tc::tf32_rn(v[1]), tc::tf32_rn(v[2]), tc::tf32_rn(v[3]));
    return make_uint4(tc::pack_bf16x2(v[0], v[1]), tc::pack_bf16x2(v[2], v[3]), tc::pack_bf16x2(v[4], v[5]),
                      tc::pack_bf16x2(v[6], v[7]));
}
__device__ __forceinline__ uint32_t lo_pair(float a, float b, uint32_t hi) {
    return tc::pack_bf16x2(a - __uint_as_float(hi << 16), b - __uint_as_float(hi & 0xffff0000u));
}
__device__ __forceinline__ uint4 pack_lo(const float *v, uint4 hi) {
    return make_uint4(lo_pair(v[0], v[1], hi.x), lo_pair(v[2], v[3], hi.y), lo_pair(v[4], v[5], hi.z),
                      lo_pair(v[6], v[7], hi.w));
}

// Operand form of slot k: the DP x (DP + X) matrix [W_k | -b_k | 0], X = 16
// bf16 or 8 tf32 elements (two extra 16-byte K groups), so the MMA yields
// z = W_k (x - c) - b_k directly against samples extended by a constant 1.
// Slots are grouped in chunks of `chunk` consecutive slots; chunk g holds
// NPART parts of KGX = KG + 2 K groups: part p, K group q, slot kk, row j at
//   g * NPART*chunk*B + p * chunk*B + q * chunk*DP*16 + kk * DP*16 + j * 16
// (B = DP*KGX*16), the shared-memory layout of one chunk.
template <int KIND, int SPLIT, int DP>
__global__ void __launch_bounds__(256) tc_prepare_kernel(const float *__restrict__ w, const float *__restrict__ loc,
                                                         int d, int first, int chunk, int cslot,
                                                         unsigned char *__restrict__ ops, float *__restrict__ center) {
    constexpr int EB = KIND == tc::kBF16 ? 2 : 4;
    constexpr int PER = 16 / EB;
    constexpr int KG = DP / PER;
    constexpr int KGX = KG + 2;
    constexpr int NPART = SPLIT == 3 ? 2 : 1;
    constexpr int LD = DP + 1;
    constexpr int B_COMP = DP * KGX * 16;
    __shared__ float ws[DP * LD];
    __shared__ float dc[DP];
    __shared__ float nb[DP];
    const int k = first + blockIdx.x;
    const float *wk = w + (size_t)k * DP * DP;
    for (int e = threadIdx.x; e < DP * DP; e += blockDim.x) ws[(e / DP) * LD + e % DP] = wk[e];
    for (int c = threadIdx.x; c < DP; c += blockDim.x) {
        const float cc = c < d ? loc[(size_t)cslot * d + c] : 0.f;
        dc[c] = c < d ? loc[(size_t)k * d + c] - cc : 0.f;
        if (blockIdx.x == 0) center[c] = cc;
    }
    __syncthreads();
    // -b_k = -W_k (mu_k - c) in FP32
    for (int j = threadIdx.x; j < DP; j += blockDim.x) {
        float acc = 0.f;
        for (int c = 0; c < d; ++c) acc = fmaf(ws[j * LD + c], dc[c], acc);
        nb[j] = -acc;
    }
    __syncthreads();
    // chunk-contiguous: the operands of slots first + g*chunk .. are one block
    // laid out as the MMA reads them (part, K group, slot in chunk, row)
    const int g = (int)blockIdx.x / chunk, kk = (int)blockIdx.x % chunk;
    unsigned char *okp = ops + (size_t)g * NPART * chunk * B_COMP + (size_t)kk * DP * 16;
    for (int e = threadIdx.x; e < KGX * DP; e += blockDim.x) {
        const int q = e / DP, j = e - q * DP;
        float v[PER];
#pragma unroll
        for (int m = 0; m < PER; ++m)
            v[m] = q < KG ? ws[j * LD + q * PER + m] : (q == KG && m == 0 ? nb[j] : 0.f);
        const uint4 hi = pack_hi<KIND>(v);
        const size_t off = (size_t)q * chunk * DP * 16 + (size_t)j * 16;
        *reinterpret_cast<uint4 *>(okp + off) = hi;
        if (NPART == 2) *reinterpret_cast<uint4 *>(okp + (size_t)chunk * B_COMP + off) = pack_lo(v, hi);
    }
}

struct TcParams {
    int d, mode, family, den_kind, fixed_slot;
    int first_slot, last_slot, chunk, nchunks, ntiles, raw_stages, bring;
    int64_t n;
    const float *x;
    const unsigned char *ops;
    const float *center;
    const float *lognorm, *coef, *dofs;
    const int32_t *group;
    float *out_logden, *out_generating, *lognum;
    uint64_t *failures;
    int64_t index_base;
    int *error;
};

// Warp roles of mixture_tc_kernel.
constexpr int kConvWarps = 8;  // stage sample tiles and build the A operand
constexpr int kEpiWarps = 4;   // one per TMEM lane quadrant
constexpr int kConvThreads = 32 * kConvWarps;
constexpr int kFirstEpiWarp = 1 + kConvWarps;
constexpr int kTcThreads = 32 * (1 + kConvWarps + kEpiWarps);
constexpr int kBRing = 3;      // operand buffers in flight when a tile needs several chunks

// NOB: one component centred at its own location, whose offset column
// -W (mu - c) is therefore zero: the MMAs run over the coordinates' K groups
// only (K = DP instead of DP + 16), and three A buffers fit.
template <int KIND, int SPLIT, int DP, bool DIRECT, bool NOB>
__global__ void __launch_bounds__(kTcThreads, 1) mixture_tc_kernel(TcParams p) {
    constexpr int EB = KIND == tc::kBF16 ? 2 : 4;
    constexpr int PER = 16 / EB;              // elements per 16-byte K group
    constexpr int KG = DP / PER;              // K groups of the sample coordinates
    constexpr int KGB = KG + 2;               // operand form: plus the offset column and padding
    constexpr int KGX = NOB ? KG : KGB;       // K groups the MMAs read
    constexpr int QH = KG / 2;                // K groups converted per thread (two threads per row)
    constexpr int NPART = SPLIT == 3 ? 2 : 1;
    constexpr int RS = DP + 4;                // padded raw row (floats): conflict-free row reads
    constexpr int RAW_BYTES = kTcTile * RS * 4;
    constexpr int A_PART = kTcTile * KGX * 16;
    constexpr int B_COMP = DP * KGB * 16;
    constexpr int KSTEPS = KGX / 2;           // MMA K slices of 32 bytes
    constexpr uint32_t LBO_A = kTcTile * 16;
    const int chunk = p.chunk, nchunks = p.nchunks, S = p.raw_stages;
    // one component chunk: A double-buffered, the chunk's operands loaded once;
    // several chunks: one A buffer (a tile is converted once per nchunks items)
    // and a ring of kBRing operand buffers filled kBRing - 1 items ahead
    const int nbufA = nchunks > 1 ? 1 : NOB ? 3 : 2;
    const int nbufB = nchunks > 1 ? p.bring : 1;
    const uint32_t LBO_B = (uint32_t)(chunk * DP * 16);
    const uint32_t CHUNK_BYTES = (uint32_t)(NPART * chunk * B_COMP);

    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *s_raw = smem;
    unsigned char *s_a = s_raw + (size_t)S * RAW_BYTES;
    unsigned char *s_b = s_a + (size_t)nbufA * NPART * A_PART;
    float *s_c = reinterpret_cast<float *>(s_b + (size_t)nbufB * CHUNK_BYTES);
    __shared__ __align__(8) uint64_t a_full[3], a_empty[3], b_full[kBRing], b_empty[kBRing], d_full[2], d_empty[2];
    __shared__ uint32_t tmem_base;
    __shared__ volatile int abort_flag;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int NW = chunk * DP;  // TMEM columns of one accumulator
    const uint32_t ncols = 2 * NW <= 32 ? 32 : 2 * NW <= 64 ? 64 : 2 * NW <= 128 ? 128 : 2 * NW <= 256 ? 256 : 512;
    if (warp == 0) tc::tmem_alloc(&tmem_base, ncols);
    if (tid == 0) {
        for (int b = 0; b < 3; ++b) {
            tc::mbar_init(&a_full[b], kConvWarps);
            tc::mbar_init(&a_empty[b], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&d_full[b], 1);
            tc::mbar_init(&d_empty[b], kEpiWarps);
        }
        for (int b = 0; b < kBRing; ++b) {
            tc::mbar_init(&b_full[b], 1);
            tc::mbar_init(&b_empty[b], 1);
        }
        tc::fence_mbar_init();
        abort_flag = 0;
    }
    for (int c = tid; c < DP; c += kTcThreads) s_c[c] = p.center[c];
    // constant K groups of the A buffers: a 1 in column DP (hi part), zeros elsewhere
    for (int e = tid; e < (NOB ? 0 : nbufA * NPART * 2 * kTcTile); e += kTcThreads) {
        const int row = e % kTcTile, g = (e / kTcTile) & 1, part = (e / (2 * kTcTile)) % NPART,
                  buf = e / (2 * kTcTile * NPART);
        const uint32_t one = KIND == tc::kTF32 ? 0x3F800000u : 0x3F80u;
        const uint32_t first = (g == 0 && part == 0) ? one : 0u;
        *reinterpret_cast<uint4 *>(s_a + (size_t)(buf * NPART + part) * A_PART + (size_t)(KG + g) * LBO_A +
                                   row * 16) = make_uint4(first, 0u, 0u, 0u);
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tmem_base;

    const int my_tiles = (p.ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
    const int J = my_tiles * nchunks;
    auto tile_of = [&](int it) -> int64_t { return (int64_t)blockIdx.x + (int64_t)it * gridDim.x; };
    auto chunk_range = [&](int ch, int &k0, int &cnt) {
        k0 = p.first_slot + ch * chunk;
        cnt = min(chunk, p.last_slot - k0 + 1);
    };
    // bounded wait that gives up at once after any role has timed out
    auto wait = [&](uint64_t *bar, uint32_t parity) -> bool {
        if (abort_flag) return false;
        if (tc::mbar_wait(bar, parity)) return true;
        atomicExch(p.error, 1);
        abort_flag = 1;
        return false;
    };

    if (warp == 0) {
        // ================= issuer: component operands and MMAs =================
        int b_issued = 0, b_waited = 0;
        // the chunk's operands are one contiguous block in the workspace, laid
        // out as in shared memory: one bulk copy per item
        auto issue_b = [&](int j) {
            const int buf = j % nbufB;
            if (lane == 0) {
                tc::mbar_arrive_expect_tx(&b_full[buf], CHUNK_BYTES);
                tc::bulk_copy_g2s(s_b + (size_t)buf * CHUNK_BYTES, p.ops + (size_t)(j % nchunks) * CHUNK_BYTES,
                                  CHUNK_BYTES, &b_full[buf]);
            }
            __syncwarp();
            ++b_issued;
        };
        // single chunk: its operands once; several: fill the ring
        for (int q = 0; q < nbufB && q < J; ++q) issue_b(q);
        for (int j = 0; j < J; ++j) {
            const int it = j / nchunks, ch = j - it * nchunks;
            const int abuf = it % nbufA;
            int ok = 1;
            if (lane == 0) {
                if (ch == 0 && !wait(&a_full[abuf], (uint32_t)((it / nbufA) & 1))) ok = 0;
                if (nchunks > 1 || j == 0) {
                    if (!wait(&b_full[j % nbufB], (uint32_t)((j / nbufB) & 1))) ok = 0;
                    else b_waited = j + 1;
                }
                if (j >= 2 && !wait(&d_empty[j & 1], (uint32_t)(((j - 2) >> 1) & 1))) ok = 0;
                tc::fence_after_sync();
                if (ok) {
                    int k0, cnt;
                    chunk_range(ch, k0, cnt);
                    const uint32_t d_tmem = tbase + (uint32_t)((j & 1) * NW);
                    const uint32_t idesc = tc::instr_desc(KIND, kTcTile, cnt * DP);
                    const uint32_t a0 = tc::smem_u32(s_a + (size_t)abuf * NPART * A_PART);
                    const uint32_t b0 = tc::smem_u32(s_b + (size_t)(j % nbufB) * CHUNK_BYTES);
#pragma unroll
                    for (int s = 0; s < KSTEPS; ++s) {
                        const uint64_t da = tc::smem_desc(a0 + s * 2 * LBO_A, LBO_A, 128);
                        const uint64_t db = tc::smem_desc(b0 + s * 2 * LBO_B, LBO_B, 128);
                        if (KIND == tc::kTF32) {
                            tc::mma_tf32(d_tmem, da, db, idesc, s > 0);
                        } else {
                            tc::mma(d_tmem, da, db, idesc, s > 0);
                            if (SPLIT == 3) {
                                const uint64_t dal = tc::smem_desc(a0 + A_PART + s * 2 * LBO_A, LBO_A, 128);
                                const uint64_t dbl = tc::smem_desc(b0 + chunk * B_COMP + s * 2 * LBO_B, LBO_B, 128);
                                tc::mma(d_tmem, dal, db, idesc, true);
                                tc::mma(d_tmem, da, dbl, idesc, true);
                            }
                        }
                    }
                }
                // commits arrive when every earlier MMA has completed, issued or not
                tc::commit(&d_full[j & 1]);
                if (nchunks > 1) tc::commit(&b_empty[j % nbufB]);
                if (ch == nchunks - 1) tc::commit(&a_empty[abuf]);
            }
            ok = __shfl_sync(0xffffffffu, ok, 0);
            // operands of item j + nbufB - 1 go into the buffer MMA j - 1 has finished with
            const int jn = j + nbufB - 1;
            if (nchunks > 1 && j >= 1 && jn < J) {
                int fine = 1;
                if (lane == 0 && !wait(&b_empty[jn % nbufB], (uint32_t)(((jn - nbufB) / nbufB) & 1))) fine = 0;
                fine = __shfl_sync(0xffffffffu, fine, 0);
                if (fine) issue_b(jn);
            }
        }
        // drain: every requested copy has landed before the CTA exits
        if (lane == 0)
            for (int q = b_waited; q < b_issued; ++q) tc::mbar_wait(&b_full[q % nbufB], (uint32_t)((q / nbufB) & 1));
    } else if (warp < kFirstEpiWarp) {
        // ================= converters: sample tiles -> A operand =================
        const int ctid = tid - 32;
        const bool vec = (p.d % 4 == 0) && ((reinterpret_cast<uintptr_t>(p.x) & 15) == 0);
        auto issue_raw = [&](int it) {
            if (it < my_tiles) {
                const int64_t row0 = tile_of(it) * kTcTile;
                const int rows = (int)min((int64_t)kTcTile, p.n - row0);
                float *dst = reinterpret_cast<float *>(s_raw + (size_t)(it % S) * RAW_BYTES);
                const float *src = p.x + row0 * p.d;
                if (vec && p.d == DP) {
                    constexpr int Q4 = DP / 4;
                    const int total = rows * Q4;
                    for (int e = ctid; e < total; e += kConvThreads) {
                        const int r = e / Q4, c4 = e % Q4;
                        tc::cp_async16(dst + r * RS + c4 * 4, src + (size_t)e * 4);
                    }
                } else if (vec) {
                    const int q4 = p.d >> 2, total = rows * q4;
                    for (int e = ctid; e < total; e += kConvThreads) {
                        const int r = e / q4, c4 = e - r * q4;
                        tc::cp_async16(dst + r * RS + c4 * 4, src + (size_t)r * p.d + c4 * 4);
                    }
                } else {
                    const int total = rows * p.d;
                    for (int e = ctid; e < total; e += kConvThreads) {
                        const int r = e / p.d, c = e - r * p.d;
                        tc::cp_async4(dst + r * RS + c, src + (size_t)r * p.d + c);
                    }
                }
            }
            tc::cp_async_commit();
        };
        for (int s = 0; s < S; ++s) issue_raw(s);
        const int row = ctid & (kTcTile - 1), half = ctid >> 7;
        constexpr int HV = DP / 8;  // float4s of this thread's half row
        for (int it = 0; it < my_tiles; ++it) {
            const int64_t i = tile_of(it) * kTcTile + row;
            const bool active = i < p.n;
            // DIRECT (no staged tile): this thread's half row straight from
            // global memory into registers, issued before the A-buffer wait so
            // its latency overlaps the previous tile's MMAs
            float4 gv[DIRECT ? HV : 1];
            if constexpr (DIRECT) {
#pragma unroll
                for (int u = 0; u < HV; ++u) {
                    const int c = half * (DP / 2) + 4 * u;
                    if (active && vec && c + 3 < p.d) {
                        gv[u] = *reinterpret_cast<const float4 *>(p.x + i * p.d + c);
                    } else {
                        const float *xr = p.x + i * p.d;
                        gv[u] = make_float4(active && c < p.d ? xr[c] : 0.f, active && c + 1 < p.d ? xr[c + 1] : 0.f,
                                            active && c + 2 < p.d ? xr[c + 2] : 0.f,
                                            active && c + 3 < p.d ? xr[c + 3] : 0.f);
                    }
                }
            } else {
                if (S == 1) tc::cp_async_wait<0>();
                else if (S == 2) tc::cp_async_wait<1>();
                else tc::cp_async_wait<2>();
                tc::named_sync(1, kConvThreads);
            }
            bool ok = true;
            const int abuf = it % nbufA;
            if (it >= nbufA) {
                if (lane == 0) ok = wait(&a_empty[abuf], (uint32_t)(((it - nbufA) / nbufA) & 1));
                ok = __shfl_sync(0xffffffffu, (int)ok, 0) != 0;
            }
            if (ok) {
                const float *raw = S > 0 ? reinterpret_cast<const float *>(s_raw + (size_t)(it % S) * RAW_BYTES)
                                         : nullptr;
                unsigned char *a = s_a + (size_t)abuf * NPART * A_PART;
                const bool full = active && p.d == DP;
#pragma unroll
                for (int qq = 0; qq < QH; ++qq) {
                    const int q = half * QH + qq;
                    float v[PER];
#pragma unroll
                    for (int m = 0; m < PER; m += 4) {
                        const int c = q * PER + m;
                        const float4 cc = *reinterpret_cast<const float4 *>(s_c + c);
                        if constexpr (DIRECT) {
                            // gv holds zeros beyond d and for inactive rows
                            const float4 f = gv[(qq * PER + m) / 4];
                            v[m] = (active && c < p.d) ? f.x - cc.x : 0.f;
                            v[m + 1] = (active && c + 1 < p.d) ? f.y - cc.y : 0.f;
                            v[m + 2] = (active && c + 2 < p.d) ? f.z - cc.z : 0.f;
                            v[m + 3] = (active && c + 3 < p.d) ? f.w - cc.w : 0.f;
                        } else if (full) {
                            const float4 f = *reinterpret_cast<const float4 *>(raw + row * RS + c);
                            v[m] = f.x - cc.x;
                            v[m + 1] = f.y - cc.y;
                            v[m + 2] = f.z - cc.z;
                            v[m + 3] = f.w - cc.w;
                        } else {
                            float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
                            if (active) f = *reinterpret_cast<const float4 *>(raw + row * RS + c);
                            v[m] = (active && c < p.d) ? f.x - cc.x : 0.f;
                            v[m + 1] = (active && c + 1 < p.d) ? f.y - cc.y : 0.f;
                            v[m + 2] = (active && c + 2 < p.d) ? f.z - cc.z : 0.f;
                            v[m + 3] = (active && c + 3 < p.d) ? f.w - cc.w : 0.f;
                        }
                    }
                    const uint4 hi = pack_hi<KIND>(v);
                    *reinterpret_cast<uint4 *>(a + (size_t)q * LBO_A + row * 16) = hi;
                    if (NPART == 2)
                        *reinterpret_cast<uint4 *>(a + A_PART + (size_t)q * LBO_A + row * 16) = pack_lo(v, hi);
                }
            }
            tc::fence_proxy_async();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&a_full[it % nbufA]);
            if (!DIRECT) {
                tc::named_sync(1, kConvThreads);  // the stage is consumed: refill it
                issue_raw(it + S);
            }
        }
        tc::cp_async_wait_all();
    } else {
        // ================= epilogue: radial densities and the log-sum-exp =================
        const int qd = warp & 3;
        const int erow = 32 * qd + lane;
        const int ggen = (p.den_kind == ISSM_DENOM_PARTIAL) ? p.group[p.fixed_slot] : 0;
        LseState<float> lse;
        float gen_lq = 0.f, last_lq = 0.f, prev_ln = 0.f;
        for (int j = 0; j < J; ++j) {
            const int it = j / nchunks, ch = j - it * nchunks;
            const int64_t i = tile_of(it) * kTcTile + erow;
            if (ch == 0 && p.mode == 1) prev_ln = i < p.n ? p.lognum[i] : 0.f;
            const bool ok = __all_sync(0xffffffffu, wait(&d_full[j & 1], (uint32_t)((j >> 1) & 1)));
            tc::fence_after_sync();
            if (ok) {
                int k0, cnt;
                chunk_range(ch, k0, cnt);
                const uint32_t lane_base = tbase + ((uint32_t)(32 * qd) << 16) + (uint32_t)((j & 1) * NW);
                for (int kk = 0; kk < cnt; ++kk) {
                    // a component's DP columns in one round trip (all loads, then one wait)
                    float v[DP];
                    if constexpr (DP == 64) tc::tmem_ld64(lane_base + (uint32_t)(kk * DP), v);
                    else if constexpr (DP == 32) tc::tmem_ld32(lane_base + (uint32_t)(kk * DP), v);
                    else tc::tmem_ld16(lane_base + (uint32_t)(kk * DP), v);
                    float r2a = 0.f, r2b = 0.f;
#pragma unroll
                    for (int q = 0; q < DP; q += 2) {
                        r2a = fmaf(v[q], v[q], r2a);
                        r2b = fmaf(v[q + 1], v[q + 1], r2b);
                    }
                    const float r2 = r2a + r2b;
                    const int k = k0 + kk;
                    float lq;
                    if (p.family == ISSM_GAUSSIAN) {
                        lq = p.lognorm[k] - 0.5f * r2;
                    } else {
                        const float nu = p.dofs[k];
                        lq = p.lognorm[k] - (nu + (float)p.d) * 0.5f * log1pf(r2 / nu);
                    }
                    bool member = true;
                    if (p.den_kind == ISSM_DENOM_GENERATING) member = (k == p.fixed_slot);
                    else if (p.den_kind == ISSM_DENOM_PARTIAL) member = (p.group[k] == ggen);
                    if (k == p.fixed_slot) gen_lq = lq;
                    last_lq = lq;
                    if (member) lse.add((p.coef ? p.coef[k] : 0.f) + lq);
                }
            }
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&d_empty[j & 1]);
            if (ch != nchunks - 1) continue;
            if (ok && i < p.n) {
                if (p.mode == 1) {
                    uint16_t reason = isnan(last_lq) ? ISSM_REASON_PROPOSAL_INVALID : 0;
                    if (!reason) {
                        const float v = logaddexp(prev_ln, p.coef[p.first_slot] + last_lq);
                        if (isnan(v) || v == -INFINITY) reason = ISSM_REASON_PROPOSAL_INVALID;
                        else p.lognum[i] = v;
                    }
                    if (reason) record_failure(p.failures, p.index_base + i + 1, 0, reason);
                } else {
                    float den = lse.value();
                    const bool bad = isnan(gen_lq) || gen_lq == -INFINITY || isnan(den) || den == -INFINITY;
                    if (bad) {
                        record_failure(p.failures, p.index_base + i + 1, 0, ISSM_REASON_PROPOSAL_INVALID);
                        den = -INFINITY;
                    }
                    p.out_logden[i] = den;
                    if (p.out_generating) p.out_generating[i] = bad ? -INFINITY : gen_lq;
                }
            }
            lse = LseState<float>();
            gen_lq = 0.f;
            last_lq = 0.f;
        }
    }
    // ---- every role is done; in-flight MMAs have completed before TMEM is freed ----
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0 && abort_flag && J > 0) tc::mbar_wait(&d_full[(J - 1) & 1], (uint32_t)(((J - 1) >> 1) & 1));
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, ncols);
}

// W_k = L_k^-1 (FP32) for slots first..first+count-1, written DP x DP
// row-major (row j = W_k[j, :]) with zero padding; one CTA of 256 per slot.
template <typename T>
__global__ void __launch_bounds__(256) invert_factors_kernel(const T *__restrict__ L, int d, int DP, int first,
                                                             float *__restrict__ w) {
    constexpr int LD = 65;
    __shared__ float Ls[64 * LD];
    __shared__ float Ws[64 * LD];
    const int k = first + blockIdx.x;
    const T *Lk = L + (size_t)k * d * d;
    // column-major source: element (r, c) at r + c d
    for (int e = threadIdx.x; e < d * d; e += blockDim.x) {
        const int r = e % d, c = e / d;
        Ls[r * LD + c] = (float)Lk[e];
    }
    __syncthreads();
    invert_lower_f32(Ls, Ws, d, LD);
    float *wk = w + (size_t)k * DP * DP;
    for (int e = threadIdx.x; e < DP * DP; e += blockDim.x) {
        const int j = e / DP, c = e % DP;
        wk[e] = (j < d && c < d) ? Ws[j * LD + c] : 0.f;
    }
}

int invert_factors(const issm_bank *bk, int first, int count, float *out, cudaStream_t stream) {
    const int d = bk->dim;
    if (d > 64) return ISSM_E_UNSUPPORTED;
    const int DP = d <= 16 ? 16 : d <= 32 ? 32 : 64;
    if (count <= 0) return 0;
    if (bk->dtype == ISSM_F32) {
        { invert_factors_kernel<float><<<count, 256, 0, stream>>>((const float *)bk->scales, d, DP, first, out);
          note_launch(); }
    } else {
        { invert_factors_kernel<double><<<count, 256, 0, stream>>>((const double *)bk->scales, d, DP, first, out);
          note_launch(); }
    }
    return (int)cudaGetLastError();
}

// Workspace: operand forms (K + 256/DP - 1) x DP * (4 DP + 64) bytes (room
// for the last, partial chunk) | centre (256 bytes) | inverse factors
// K x DP * DP floats (only when the bank has none).
static int dp_of(int d) { return d <= 16 ? 16 : d <= 32 ? 32 : 64; }
static size_t ops_slot_bytes(int DP) { return (size_t)DP * (4 * DP + 64); }
static size_t ops_bytes(int k, int DP) { return (size_t)(k + 256 / DP - 1) * ops_slot_bytes(DP); }

size_t tc_workspace_bytes(int k, int d) {
    const int DP = dp_of(d);
    return ops_bytes(k, DP) + 256 + (size_t)k * DP * DP * 4 + 64;
}

template <int KIND, int SPLIT, int DP>
static int launch_tc(TcParams p, const float *w, const float *loc, int cslot, unsigned char *ops, float *center,
                     cudaStream_t stream) {
    constexpr int EB = KIND == tc::kBF16 ? 2 : 4;
    constexpr int KGX = DP * EB / 16 + 2;
    constexpr int NPART = SPLIT == 3 ? 2 : 1;
    constexpr size_t RAW_BYTES = (size_t)kTcTile * (DP + 4) * 4;
    constexpr size_t A_PART = (size_t)kTcTile * KGX * 16;
    constexpr size_t A_PART_NOB = (size_t)kTcTile * (KGX - 2) * 16;
    constexpr size_t B_COMP = (size_t)DP * KGX * 16;
    static_assert(NPART * B_COMP <= (size_t)DP * (4 * DP + 64), "operand form exceeds its workspace slot");
    const int nslots = p.last_slot - p.first_slot + 1;
    // one component centred at its own location: no offset column
    const bool nob = nslots == 1 && cslot == p.first_slot;
    // largest chunk (<= 256 TMEM columns) whose buffers fit: one chunk keeps
    // three staged tiles and two A buffers; several chunks keep one A buffer
    // and a ring of kBRing chunk buffers, with one staged tile or none
    int chunk = min(nslots, 256 / DP), nch = 1, stages = 1, bring = kBRing;
    size_t smem = 0;
    for (; chunk >= 1; --chunk) {
        nch = (nslots + chunk - 1) / chunk;
        if (nch == 1) {
            stages = 3;
            smem = stages * RAW_BYTES + (nob ? 3 * NPART * A_PART_NOB : 2 * NPART * A_PART) +
                   (size_t)NPART * chunk * B_COMP + (size_t)DP * 4;
        } else {
            // a staged tile if it fits beside a kBRing-deep operand ring; else
            // the converters read their rows from global memory (no staged
            // tile), with a kBRing- or 2-deep ring, which leaves room for
            // larger chunks (fewer, wider MMA items per tile)
            const size_t base = NPART * A_PART + (size_t)DP * 4, cb = (size_t)NPART * chunk * B_COMP;
            bring = kBRing;
            stages = RAW_BYTES + base + kBRing * cb <= kTcMaxSmem ? 1 : 0;
            if (stages == 0 && base + kBRing * cb > kTcMaxSmem) bring = 2;
            smem = stages * RAW_BYTES + base + bring * cb;
        }
        if (smem <= kTcMaxSmem) break;
    }
    if (chunk < 1) return ISSM_E_UNSUPPORTED;
    p.chunk = chunk;
    p.nchunks = nch;
    p.raw_stages = stages;
    p.bring = bring;
    { tc_prepare_kernel<KIND, SPLIT, DP><<<nslots, 256, 0, stream>>>(w, loc, p.d, p.first_slot, chunk, cslot, ops,
                                                                       center);
      note_launch(); }
    // DIRECT (no staged tile; converters read rows from global memory) is a
    // separate instantiation so the staged form keeps its registers
    auto kern = stages == 0 ? mixture_tc_kernel<KIND, SPLIT, DP, true, false>
                : nob && nch == 1 ? mixture_tc_kernel<KIND, SPLIT, DP, false, true>
                                  : mixture_tc_kernel<KIND, SPLIT, DP, false, false>;
    const int st = allow_dynamic_smem((const void *)kern);
    if (st) return st;
    int occ = 1;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kTcThreads, smem);
    if (e != cudaSuccess) return (int)e;
    const int nw2 = 2 * chunk * DP;
    const int ncols = nw2 <= 32 ? 32 : nw2 <= 64 ? 64 : nw2 <= 128 ? 128 : nw2 <= 256 ? 256 : 512;
    occ = max(1, min(occ, 512 / ncols));  // TMEM allocations never wait
    p.ntiles = (int)((p.n + kTcTile - 1) / kTcTile);
    const int blocks = min(p.ntiles, device_sms() * occ);
    if (blocks < 1) return 0;
    { kern<<<blocks, kTcThreads, smem, stream>>>(p); note_launch(); }
    return (int)cudaGetLastError();
}

// precision: ISSM_PREC_TF32 or ISSM_PREC_BF16 (split x3)
int tc_mixture(const issm_bank *bk, const issm_denominator *den, int mode, int first, int last,
               const void *x, int64_t n, const int32_t *slots, int fixed_slot, const void *coef,
               void *out_logden, void *out_generating, void *lognum, uint64_t *failures, int64_t index_base,
               int precision, void *ws, size_t ws_bytes, int *error, cudaStream_t stream) {
    const int d = bk->dim;
    if (bk->dtype != ISSM_F32 || bk->scale_kind != ISSM_SCALE_FACTOR || d > 64) return ISSM_E_UNSUPPORTED;
    if (slots != nullptr) return ISSM_E_UNSUPPORTED;  // one centre per launch
    const int DP = dp_of(d);
    const int K = bk->count;
    if (ws_bytes < tc_workspace_bytes(K, d)) return ISSM_E_WORKSPACE;
    unsigned char *ops = (unsigned char *)ws;
    float *center = (float *)(ops + ops_bytes(K, DP));
    float *winv = (float *)((unsigned char *)center + 256);
    const int den_kind = den ? den->kind : ISSM_DENOM_FULL;
    // only the generating slot contributes to a generating-only denominator
    if (mode == 0 && den_kind == ISSM_DENOM_GENERATING) first = last = fixed_slot;
    const float *w = bk->inverse_factors;
    if (!w) {
        const int st = invert_factors(bk, first, last - first + 1, winv, stream);
        if (st) return st;
        w = winv;
    }
    const int cslot = (mode == 1) ? first : fixed_slot;
    TcParams p{};
    p.d = d; p.mode = mode; p.family = bk->family; p.den_kind = den_kind; p.fixed_slot = fixed_slot;
    p.first_slot = first; p.last_slot = last;
    p.n = n; p.x = (const float *)x; p.ops = ops; p.center = center;
    p.lognorm = (const float *)bk->lognormalizers; p.coef = (const float *)coef; p.dofs = (const float *)bk->dofs;
    p.group = den ? den->group_of_slot : nullptr;
    p.out_logden = (float *)out_logden; p.out_generating = (float *)out_generating;
    p.lognum = (float *)lognum; p.failures = failures; p.index_base = index_base; p.error = error;
    const float *loc = (const float *)bk->locations;
    const bool tf32 = precision == ISSM_PREC_TF32;
    if (DP == 16)
        return tf32 ? launch_tc<tc::kTF32, 1, 16>(p, w, loc, cslot, ops, center, stream)
                    : launch_tc<tc::kBF16, 3, 16>(p, w, loc, cslot, ops, center, stream);
    if (DP == 32)
        return tf32 ? launch_tc<tc::kTF32, 1, 32>(p, w, loc, cslot, ops, center, stream)
                    : launch_tc<tc::kBF16, 3, 32>(p, w, loc, cslot, ops, center, stream);
    return tf32 ? launch_tc<tc::kTF32, 1, 64>(p, w, loc, cslot, ops, center, stream)
                : launch_tc<tc::kBF16, 3, 64>(p, w, loc, cslot, ops, center, stream);
}

}  // namespace issm
