// tcgen05.cuh — inline-PTX helpers for the 5th-generation tensor cores of
// sm_103a: tensor-memory (TMEM) allocation, shared-memory matrix descriptors
// for the no-swizzle K-major canonical layout, the instruction descriptor of
// kind::f16 / kind::tf32, MMA issue and commit, bounded mbarrier waits, and
// TMEM -> register loads.
//
// Canonical no-swizzle K-major tile (rows = M or N, columns = K):
//   the tile is a grid of "core matrices" of 8 rows x 16 bytes stored as 128
//   contiguous bytes (row r at byte 16 r). Core matrix (row group g, K group
//   q) sits at byte (g * KG + q) * 128, KG = K * elem_bytes / 16. So the
//   leading byte offset (next core matrix along K) is 128 and the stride byte
//   offset (next 8-row group) is KG * 128. One MMA instruction consumes 32
//   bytes of K (16 bf16 or 8 tf32 elements) = two K-adjacent core matrices;
//   successive K slices advance the descriptor start address by 256 bytes.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace issm {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (row, k) inside a canonical no-swizzle K-major tile
__device__ __forceinline__ uint32_t kmajor_offset(int row, int k, int k_groups, int elem_bytes) {
    const int per = 16 / elem_bytes;  // elements per core-matrix row
    return (uint32_t)((((row >> 3) * k_groups + k / per) << 7) + ((row & 7) << 4) + (k % per) * elem_bytes);
}

// Row-contiguous variant of the same canonical layout: for each 16-byte K
// group q the tile's `rows` rows are stored consecutively (row r at 16 r), so
// core matrix (row group g, K group q) sits at q * rows * 16 + g * 128: the
// leading byte offset is rows * 16 and the stride byte offset 128. Writing one
// K group for 32 consecutive rows touches 512 contiguous bytes (no bank
// conflicts), and one K slice of 32 bytes advances the start by 2 * rows * 16.
__device__ __forceinline__ uint32_t rowgroup_offset(int row, int k, int rows, int elem_bytes) {
    const int per = 16 / elem_bytes;
    return (uint32_t)((k / per) * rows * 16 + row * 16 + (k % per) * elem_bytes);
}

// MN-major (16-bit elements): element (row, k) of a tile with K extent
// `kext`; each group of 8 rows stores its K elements consecutively, 16 bytes
// (the 8 rows) per K index, so one sample's 8 coordinates form one 16-byte
// chunk and 8 consecutive K indices form one 128-byte core matrix.
__device__ __forceinline__ uint32_t mn_offset(int row, int k, int kext) {
    return (uint32_t)((row >> 3) * kext * 16 + k * 16 + (row & 7) * 2);
}

// 64-bit shared-memory matrix descriptor (version 1, no swizzle).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo_bytes, uint32_t sbo_bytes) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)((lbo_bytes >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo_bytes >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
    // base offset 0, LBO mode 0, layout type 0 (no swizzle)
    return d;
}

enum Kind { kBF16 = 1, kTF32 = 2 };
// instruction-descriptor bits: A and B MN-major ("transposed") instead of K-major
constexpr uint32_t kMajorMN = (1u << 15) | (1u << 16);

// Instruction descriptor: D = F32, A/B format, both K-major, N >> 3, M >> 4.
__host__ __device__ constexpr uint32_t instr_desc(int fmt, int m, int n) {
    return (1u << 4) | ((uint32_t)fmt << 7) | ((uint32_t)fmt << 10) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// make generic-proxy shared-memory writes visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Whole warp: allocate `ncols` TMEM columns (power of two >= 32); the base
// address is written to *dst_smem.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// One thread: D[tmem] (+)= A[smem] * B[smem]^T
__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                    bool accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"((uint32_t)accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         bool accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"((uint32_t)accumulate)
        : "memory");
}

// One thread: the mbarrier at `bar` receives one arrival when every
// previously issued tcgen05 op of this thread has completed.
__device__ __forceinline__ void commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Bounded wait for the phase with parity `phase` to complete. Returns false
// after `limit` polls or about one second of SM clock (the caller records an
// error and unwinds; no trap).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t phase, uint32_t limit = 1u << 22) {
    const uint32_t addr = smem_u32(bar);
    const long long t0 = clock64();
    for (uint32_t i = 0; i < limit; ++i) {
        if ((i & 255) == 255 && clock64() - t0 > 2000000000ll) return false;
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(addr), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Warp-collective TMEM -> registers: thread t of the warp reads TMEM lane
// (lane base + t) and 16 consecutive 32-bit columns starting at taddr.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ---- asynchronous copies ------------------------------------------------------
// 16-byte global -> shared copy that bypasses L1 (both addresses 16-byte aligned)
__device__ __forceinline__ void cp_async16(void *dst_smem, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst_smem)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void *dst_smem, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst_smem)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// One arrival on the mbarrier (release at CTA scope).
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Named barrier `id` (1..15) over `count` threads (a multiple of 32).
__device__ __forceinline__ void named_sync(int id, int count) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// Expect `bytes` of bulk-copy completions on the mbarrier, and arrive once.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
// Bulk global -> shared copy (addresses 16-byte aligned, size a multiple of
// 16) whose completion is counted on the mbarrier in bytes.
__device__ __forceinline__ void bulk_copy_g2s(void *dst_smem, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst_smem)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Tiled 2-D tensor copy global -> shared through a tensor map (this GPU's own
// memory, no multicast); completion counted on the mbarrier in bytes. x is the
// inner (element) coordinate and must be a multiple of 16 bytes; y the row.
__device__ __forceinline__ void tma_load_2d(void *dst_smem, const void *tmap, int x, int y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst_smem)), "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Shared-memory address of the 16-byte chunk holding coordinates c .. c + 3
// (c a multiple of 4) of `row` in a tile staged by 128-byte-swizzled tensor
// copies of 32-float boxes: box c / 32 of 128 rows x 128 bytes, chunk
// (c / 4) % 8 of the row XOR (row % 8).
__device__ __forceinline__ const float *swizzled_row_chunk(const unsigned char *stage, int row, int c) {
    const int c4 = c >> 2;
    return reinterpret_cast<const float *>(stage + (size_t)(c4 >> 3) * 16384 + (size_t)row * 128 +
                                           ((((c4 & 7) ^ (row & 7))) << 4));
}

// Two FP32 values rounded to nearest-even bf16 and packed: a in the low half,
// b in the high half (cvt.rn.bf16x2 puts its first source in the high half).
__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    uint32_t r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(b), "f"(a));
    return r;
}
// FP32 rounded to nearest-even tf32 (low 13 mantissa bits cleared).
__device__ __forceinline__ uint32_t tf32_rn(float f) {
    uint32_t r;
    asm("cvt.rn.tf32.f32 %0, %1;" : "=r"(r) : "f"(f));
    return r;
}

// Warp-collective TMEM -> registers of 32 or 64 consecutive columns: every
// load is issued before one tcgen05.wait::ld, in a single asm statement so no
// use of the registers can be scheduled before the wait.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%32];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%33];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr), "r"(taddr + 16u)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, float (&v)[64]) {
    uint32_t r[64];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%64];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%65];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47}, [%66];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%67];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
        : "r"(taddr), "r"(taddr + 16u), "r"(taddr + 32u), "r"(taddr + 48u)
        : "memory");
#pragma unroll
    for (int i = 0; i < 64; ++i) v[i] = __uint_as_float(r[i]);
}

// 8-column variant of tmem_ld16.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint16_t bf16_bits(float f) {
    // round to nearest even (finite inputs); NaN stays NaN
    uint32_t u = __float_as_uint(f);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

}  // namespace tc
}  // namespace issm
