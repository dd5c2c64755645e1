// mlp_tc.cuh -- the learned sensor's network on the 5th-generation tensor cores: the two 64x64
// hidden layers of 128 cells at a time as tcgen05.mma (kind::tf32) with the accumulators in
// tensor memory, in 3xTF32 form (a = a_hi + a_lo with a_hi the TF32 truncation; A*B ~ A_hi*B_hi +
// A_hi*B_lo + A_lo*B_hi accumulated in FP32), so the products keep FP32 accuracy.
//
// Operands live in shared memory in the K-major canonical layout without swizzle: 8-row x
// 16-byte core matrices, the 16 core matrices of a row group along K contiguous (leading-byte
// offset 128 B), row groups 2048 B apart (stride-byte offset). One thread issues the MMAs; an
// mbarrier signals their completion; each warp reads its lane quarter of the accumulator with
// tcgen05.ld.
#pragma once

#include <cstdint>
#include <cstring>

#include "async.cuh"
#include "device.cuh"

namespace plens_gpu {
namespace tc {

constexpr int kRows = 128;                       // cells per tile (MMA M)
constexpr int kK = 64, kN = 64;                  // layer width (MMA K and N)
constexpr int kMatA = kRows * kK * 4;            // bytes of one A operand (hi or lo)
constexpr int kMatB = kN * kK * 4;               // bytes of one B operand
constexpr uint32_t kTmemCols = 64;               // FP32 accumulator 128 lanes x 64 columns

// Cells per tile of the one-tile-per-SM kernels (the tensor-core indicators): the fewest tiles
// that fill the SMs evenly -- ceil(nc / (nsm * waves)) rows with waves = ceil(nc / (nsm * kRows))
// -- so that a mesh of fewer than nsm x 128 cells spreads over every SM instead of leaving some
// idle (14,400 cells: 152 tiles of 95 instead of 113 of 128). The rows past a tile's cells are
// zero operands.
inline int tile_rows(int64_t nc, int nsm)
{
    if (nc < 1 || nsm < 1) return kRows;
    const int64_t cap = (int64_t)nsm * kRows, waves = (nc + cap - 1) / cap;
    const int64_t per = (nc + (int64_t)nsm * waves - 1) / ((int64_t)nsm * waves);
    return (int)(per < 1 ? 1 : (per > kRows ? kRows : per));
}

// float offset of element (row r, k) in the canonical K-major no-swizzle layout of a 64-wide K
__host__ __device__ __forceinline__ int core_off(int r, int k)
{
    return (((r >> 3) * (kK / 4) + (k >> 2)) * 32) + (r & 7) * 4 + (k & 3);
}

__device__ __forceinline__ uint32_t s_addr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// shared-memory matrix descriptor: start address, LBO = 128 B (K direction), SBO = 2048 B
// (8-row groups), descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t desc_kmajor(const void* p)
{
    const uint32_t a = s_addr(p);
    uint64_t d = (uint64_t)((a >> 4) & 0x3FFFu);
    d |= (uint64_t)(128u >> 4) << 16;
    d |= (uint64_t)(2048u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// instruction descriptor: D FP32, A and B TF32, both K-major, N = 64, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kN >> 3) << 17) | ((uint32_t)(kRows >> 4) << 24);

__device__ __forceinline__ void tmem_alloc(uint32_t* dst) // one full warp
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(s_addr(dst)), "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr) // the allocating warp
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(kTmemCols) : "memory");
}
__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(s_addr(bar))
                 : "memory");
}
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_smem_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 32 lanes x 32 consecutive FP32 columns of the accumulator (this thread: its lane's 32 values)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// 32 lanes x 16 consecutive FP32 columns of the accumulator
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
        "[%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__host__ __device__ __forceinline__ float tf32_hi(float x)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(__float_as_uint(x) & 0xffffe000u);
#else
    uint32_t u;
    memcpy(&u, &x, 4);
    u &= 0xffffe000u;
    float y;
    memcpy(&y, &u, 4);
    return y;
#endif
}

// one layer of 128 rows: D = A x B^T in 3xTF32 (24 MMAs of K = 8), issued by one thread
__device__ __forceinline__ void layer_mma(uint32_t d, const float* a_hi, const float* a_lo, const float* b_hi,
                                          const float* b_lo)
{
#pragma unroll
    for (int s = 0; s < kK / 8; ++s) {
        const int off = s * 64;  // two core matrices along K = 256 B = 64 floats
        mma_tf32(d, desc_kmajor(a_hi + off), desc_kmajor(b_hi + off), s > 0);
        mma_tf32(d, desc_kmajor(a_hi + off), desc_kmajor(b_lo + off), 1);
        mma_tf32(d, desc_kmajor(a_lo + off), desc_kmajor(b_hi + off), 1);
    }
}

}  // namespace tc
}  // namespace plens_gpu
