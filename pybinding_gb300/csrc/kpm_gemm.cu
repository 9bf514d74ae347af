// Tensor-core moments matrix of the Kubo-Bastin conductivity:
//   mu += L R^H   (mu: M x M, L and R: M x I, I = rows x vectors)
// (kpm/Moments.cpp:92-101 MomentMultiplication::matrix_mul_add is the CPU form).
//
// tcgen05 kind::tf32 with a three-product split: every FP32 operand x is written as
// hi + lo with hi = tf32(x) (round to nearest, ties away) and lo = x - hi (exact), and
// each real product is hi*hi + hi*lo + lo*hi, which keeps FP32-level accuracy (the
// dropped lo*lo term and the tf32 rounding of lo are ~2^-21 of x*y). Operands are
// real/imaginary planes (row-major, K-major for the MMA), so the complex product is
//   Re += Lr.Rr^T + Li.Ri^T,   Im += Li.Rr^T - Lr.Ri^T
// with the negate-A bit of the instruction descriptor for the minus sign: 12 MMAs
// per K step into two TMEM accumulators (128 x 128 FP32 each).
//
// Pipeline per CTA (one 128 x 128 output tile, one slice of I of at most KB_MAX blocks):
//   warp 0       TMA producer: 2 or 4 tiles of 128 x 16 FP32 per stage (SWIZZLE_64B)
//   warp 1       MMA issuer (one thread) and TMEM owner
//   warps 2..9   split each landed tile in place into hi (same buffer) and lo; fold
//                every finished group accumulator into a register master; epilogue
// The tensor core's FP32 accumulation loses accuracy in proportion to the number of
// MMAs accumulated into one accumulator (measured ~2e-8 of the result per MMA, biased,
// not a random walk), so every group of `group_kb` K blocks goes into a fresh TMEM
// accumulator. Two accumulators alternate: while the tensor core fills one, the
// converter warps add the other into their FP32 registers (round to nearest). Each
// TMEM lane quarter is read by two warps (warp % 4 selects the quarter), one per half
// of the columns. At the end of the slice the registers go to mu with FP64 atomics.
// mbarriers: full/converted/empty per stage, done/free per accumulator; every wait is
// bounded by a clock limit and also ends once any CTA has flagged an error.
#include "kpm_async.cuh"
#include "kpm_internal.h"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

namespace kpm {
namespace {

constexpr int TM = 128;              // A rows per tile = TMEM lanes
constexpr int TN = 128;              // B rows per tile = accumulator columns
constexpr int TK = 16;               // FP32 per K block: one 64-byte swizzled row
constexpr int STAGES = 3;
constexpr int THREADS = 320;
constexpr int CONVERTERS = 256;      // warps 2..9, two per TMEM lane quarter
constexpr int KB_MAX = 256;          // K blocks per CTA at most (the rest goes to FP64 atomics)
constexpr uint32_t TILE_BYTES = TM * TK * 4;  // 8 KB, TM == TN

using async::mbar_arrive;
using async::mbar_drain;
using async::mbar_expect_tx;
using async::mbar_init;
using async::mbar_wait;
using async::smem_u32;

__device__ __forceinline__ void tma_load_2d(void* dst, CUtensorMap const* map, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

// UMMA shared-memory descriptor: K-major, SWIZZLE_64B (8-row atoms of 64 bytes,
// 512 bytes between 8-row groups), descriptor version 1.
__device__ __forceinline__ uint64_t desc_sw64(uint32_t addr) {
    return static_cast<uint64_t>((addr & 0x3FFFFu) >> 4) | (static_cast<uint64_t>(1) << 16) |
           (static_cast<uint64_t>(512 >> 4) << 32) | (static_cast<uint64_t>(1) << 46) |
           (static_cast<uint64_t>(4) << 61);
}

// Instruction descriptor, kind::tf32: D FP32, A/B TF32, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n, bool neg_a) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((neg_a ? 1u : 0u) << 13) | (static_cast<uint32_t>(n >> 3) << 17) |
           (static_cast<uint32_t>(m >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
        ::"r"(d), "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t u;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(u) : "f"(x));
    return __uint_as_float(u);
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

template<bool CPLX>
__global__ void __launch_bounds__(THREADS, 1)
mu_gemm_tc_kernel(const __grid_constant__ CUtensorMap map_ar, const __grid_constant__ CUtensorMap map_ai,
                  const __grid_constant__ CUtensorMap map_br, const __grid_constant__ CUtensorMap map_bi, int M,
                  int64_t I, int64_t chunk, int group_kb, double* __restrict__ mu, int* __restrict__ err) {
    constexpr int PLANES = CPLX ? 4 : 2;  // A_re, [A_im], B_re, [B_im]
    constexpr int PB = CPLX ? 2 : 1;      // first B plane
    constexpr uint32_t STAGE_BYTES = PLANES * 2 * TILE_BYTES;
    constexpr int NCOL = CPLX ? 2 * TN : TN;  // columns of one accumulator (re [, im])
    constexpr uint32_t TMEM_COLS = 2 * NCOL;  // two accumulators: 512 or 256 (a power of two)
    constexpr int HCOL = NCOL / 2;            // columns per converter warp (re or im half; 64 real)
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t{1023});
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
    uint64_t* conv = full + STAGES;
    uint64_t* empty = conv + STAGES;
    uint64_t* gdone = empty + STAGES;  // [2] an accumulator's MMAs have completed
    uint64_t* gfree = gdone + 2;       // [2] the converters have read the accumulator
    uint64_t* drain = gfree + 2;       // all MMAs of this CTA have completed
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
    auto tile = [&](int s, int plane, int hl) -> float* {
        return reinterpret_cast<float*>(smem + s * STAGE_BYTES + (plane * 2 + hl) * TILE_BYTES);
    };

    int const warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    int64_t const k_begin = static_cast<int64_t>(blockIdx.z) * chunk;
    int64_t const k_end = (k_begin + chunk < I) ? k_begin + chunk : I;
    int const nkb = k_begin < k_end ? static_cast<int>((k_end - k_begin + TK - 1) / TK) : 0;
    int const ngroups = (nkb + group_kb - 1) / group_kb;
    int const row_a = blockIdx.x * TM, row_b = blockIdx.y * TN;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(full + s, 1);
            mbar_init(conv + s, CONVERTERS);
            mbar_init(empty + s, 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(gdone + b, 1);
            mbar_init(gfree + b, CONVERTERS);
        }
        mbar_init(drain, 1);
        async::mbar_init_fence();
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    uint32_t const tmem = *tmem_slot;  // accumulator b: columns [b NCOL, (b + 1) NCOL), re then im

    if (warp == 0) {
        if (lane == 0) {  // producer
            int issued = 0;
            for (int kb = 0; kb < nkb; ++kb) {
                int const s = kb % STAGES, use = kb / STAGES;
                if (use > 0 && !mbar_wait(empty + s, (use - 1) & 1, err)) break;
                issued = kb + 1;
                mbar_expect_tx(full + s, PLANES * TILE_BYTES);
                int const k = static_cast<int>(k_begin + static_cast<int64_t>(kb) * TK);
                tma_load_2d(tile(s, 0, 0), &map_ar, full + s, k, row_a);
                if (CPLX) tma_load_2d(tile(s, 1, 0), &map_ai, full + s, k, row_a);
                tma_load_2d(tile(s, PB, 0), &map_br, full + s, k, row_b);
                if (CPLX) tma_load_2d(tile(s, 3, 0), &map_bi, full + s, k, row_b);
            }
            // copies still in flight land before the CTA leaves (already true without an error)
            for (int kb = issued - STAGES < 0 ? 0 : issued - STAGES; kb < issued; ++kb)
                mbar_drain(full + kb % STAGES, (kb / STAGES) & 1, err);
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer
            constexpr uint32_t idp = idesc_tf32(TM, TN, false);
            constexpr uint32_t idn = idesc_tf32(TM, TN, true);
            bool issued = false;
            for (int kb = 0; kb < nkb; ++kb) {
                int const s = kb % STAGES, use = kb / STAGES;
                int const g = kb / group_kb, b = g & 1;
                bool const group_start = kb % group_kb == 0;
                if (group_start && g >= 2 && !mbar_wait(gfree + b, ((g - 2) >> 1) & 1, err)) break;
                if (!mbar_wait(conv + s, use & 1, err)) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                issued = true;
                uint32_t const d_re = tmem + b * NCOL, d_im = d_re + TN;
#pragma unroll
                for (int j = 0; j < TK / 8; ++j) {  // K = 8 TF32 (32 bytes) per MMA
                    uint32_t const off = j * 32;
                    uint64_t const arh = desc_sw64(smem_u32(tile(s, 0, 0)) + off);
                    uint64_t const arl = desc_sw64(smem_u32(tile(s, 0, 1)) + off);
                    uint64_t const brh = desc_sw64(smem_u32(tile(s, PB, 0)) + off);
                    uint64_t const brl = desc_sw64(smem_u32(tile(s, PB, 1)) + off);
                    uint32_t const acc0 = (group_start && j == 0) ? 0u : 1u;
                    mma_tf32(d_re, arh, brh, idp, acc0);
                    mma_tf32(d_re, arh, brl, idp, 1u);
                    mma_tf32(d_re, arl, brh, idp, 1u);
                    if (CPLX) {
                        uint64_t const aih = desc_sw64(smem_u32(tile(s, 1, 0)) + off);
                        uint64_t const ail = desc_sw64(smem_u32(tile(s, 1, 1)) + off);
                        uint64_t const bih = desc_sw64(smem_u32(tile(s, 3, 0)) + off);
                        uint64_t const bil = desc_sw64(smem_u32(tile(s, 3, 1)) + off);
                        mma_tf32(d_re, aih, bih, idp, 1u);
                        mma_tf32(d_re, aih, bil, idp, 1u);
                        mma_tf32(d_re, ail, bih, idp, 1u);
                        mma_tf32(d_im, aih, brh, idp, acc0);
                        mma_tf32(d_im, aih, brl, idp, 1u);
                        mma_tf32(d_im, ail, brh, idp, 1u);
                        mma_tf32(d_im, arh, bih, idn, 1u);
                        mma_tf32(d_im, arh, bil, idn, 1u);
                        mma_tf32(d_im, arl, bih, idn, 1u);
                    }
                }
                mma_commit(empty + s);  // the stage is free once these MMAs have read it
                if (kb % group_kb == group_kb - 1 || kb == nkb - 1) mma_commit(gdone + b);
            }
            if (issued) {  // MMAs in flight complete before TMEM is freed (already true without an error)
                mma_commit(drain);
                mbar_drain(drain, 0, err);
            }
        }
    } else {  // converters: split landed tiles; fold finished accumulators into registers
        int const tid = threadIdx.x - 64;
        int const quarter = warp % 4;        // TMEM lanes this warp may read
        int const half = (warp - 2) / 4;     // which half of the accumulator columns
        uint32_t const lane_base = tmem + (static_cast<uint32_t>(quarter * 32) << 16) + half * HCOL;
        float mst[HCOL];
#pragma unroll
        for (int c = 0; c < HCOL; ++c) mst[c] = 0.f;
        bool ok = true;
        auto fold = [&](int g) {
            int const b = g & 1;
            if (!async::mbar_wait_warp(gdone + b, (g >> 1) & 1, err)) { ok = false; return; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int q = 0; q < HCOL / 32; ++q) {
                uint32_t r[32];
                tmem_ld32(lane_base + b * NCOL + q * 32, r);
#pragma unroll
                for (int c = 0; c < 32; ++c) mst[q * 32 + c] += __uint_as_float(r[c]);
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            mbar_arrive(gfree + b);
        };
        for (int kb = 0; kb < nkb && ok; ++kb) {
            int const s = kb % STAGES, use = kb / STAGES;
            if (!async::mbar_wait_warp(full + s, use & 1, err)) { ok = false; break; }
#pragma unroll
            for (int p = 0; p < PLANES; ++p) {
                float4* hi = reinterpret_cast<float4*>(tile(s, p, 0));
                float4* lo = reinterpret_cast<float4*>(tile(s, p, 1));
#pragma unroll
                for (int i = tid; i < static_cast<int>(TILE_BYTES / 16); i += CONVERTERS) {
                    float4 x = hi[i];
                    float4 h = make_float4(tf32_rna(x.x), tf32_rna(x.y), tf32_rna(x.z), tf32_rna(x.w));
                    hi[i] = h;
                    lo[i] = make_float4(x.x - h.x, x.y - h.y, x.z - h.z, x.w - h.w);
                }
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // visible to the tensor core
            mbar_arrive(conv + s);
            // fold the previous group once this block (the first of the next group) is handed over,
            // so that the tensor core never waits for the conversion of its next block
            if (kb % group_kb == 0 && kb > 0) fold(kb / group_kb - 1);
        }
        if (ok && ngroups > 0) fold(ngroups - 1);
        int const row = row_a + quarter * 32 + lane;
        if (ok && ngroups > 0 && row < M) {
#pragma unroll
            for (int c = 0; c < HCOL; ++c) {  // fully unrolled: mst stays in registers
                int const n = row_b + (CPLX ? c : half * HCOL + c);
                if (n < M) atomicAdd(mu + 2 * (static_cast<int64_t>(n) * M + row) + (CPLX ? half : 0),
                                     static_cast<double>(mst[c]));
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 const fn = [] {  // thread-safe one-time lookup
        cudaDriverEntryPointQueryResult q;
        void* p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        return static_cast<PFN_cuTensorMapEncodeTiled_v12000>(nullptr);
    }();
    return fn;
}

bool make_map(CUtensorMap* map, float const* base, int64_t I, int64_t rows, int64_t ld) {
    auto fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {static_cast<cuuint64_t>(I), static_cast<cuuint64_t>(rows)};
    cuuint64_t strides[1] = {static_cast<cuuint64_t>(ld) * sizeof(float)};
    cuuint32_t box[2] = {static_cast<cuuint32_t>(TK), static_cast<cuuint32_t>(TM)};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

}  // namespace

size_t mu_gemm_tc_smem(bool cplx) {
    return static_cast<size_t>(STAGES) * (cplx ? 4 : 2) * 2 * TILE_BYTES + 1024 + 256;  // + alignment, barriers
}

cudaError_t launch_mu_gemm_tc(bool cplx, float const* a_re, float const* a_im, float const* b_re, float const* b_im,
                              int64_t M, int64_t I, int64_t ld, int group_kb, double* mu, int* err, cudaStream_t s) {
    if (M < 1 || I < 1) return cudaSuccess;
    if (I > (int64_t{1} << 31) - TK || M > (int64_t{1} << 20)) return cudaErrorInvalidValue;  // int32 TMA coordinates
    // TMA: 16-byte aligned bases and row strides
    auto misaligned = [](void const* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) != 0; };
    if ((ld * 4) % 16 != 0 || ld < I || misaligned(a_re) || misaligned(b_re) || (cplx && (misaligned(a_im) || misaligned(b_im))))
        return cudaErrorInvalidValue;
    CUtensorMap mar, mai, mbr, mbi;
    if (!make_map(&mar, a_re, I, M, ld) || !make_map(&mbr, b_re, I, M, ld)) return cudaErrorInvalidValue;
    if (cplx) {
        if (!make_map(&mai, a_im, I, M, ld) || !make_map(&mbi, b_im, I, M, ld)) return cudaErrorInvalidValue;
    } else {
        mai = mar;
        mbi = mbr;
    }
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t const tiles_m = (M + TM - 1) / TM;
    int64_t const tiles = tiles_m * tiles_m;
    // slices of at most KB_MAX blocks; at least one CTA per SM; a whole number of waves when it
    // takes several
    int64_t const nkb = (I + TK - 1) / TK;
    int64_t splits = std::max<int64_t>((nkb + KB_MAX - 1) / KB_MAX, (sms + tiles - 1) / tiles);
    if (tiles * splits > sms) {
        int64_t const waves = (tiles * splits + sms - 1) / sms;
        splits = std::max<int64_t>(splits, (waves * sms) / tiles);
    }
    splits = std::min<int64_t>(splits, nkb);
    int64_t const chunk = ((nkb + splits - 1) / splits) * TK;
    splits = (I + chunk - 1) / chunk;
    if (splits > 65535) return cudaErrorInvalidValue;
    if (group_kb < 1) group_kb = 1;
    size_t const smem = mu_gemm_tc_smem(cplx);
    dim3 grid(static_cast<unsigned>(tiles_m), static_cast<unsigned>(tiles_m), static_cast<unsigned>(splits));
    cudaError_t e;
    if (cplx) {
        e = cudaFuncSetAttribute(mu_gemm_tc_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return e;
        mu_gemm_tc_kernel<true><<<grid, THREADS, smem, s>>>(mar, mai, mbr, mbi, static_cast<int>(M), I, chunk, group_kb, mu, err);
    } else {
        e = cudaFuncSetAttribute(mu_gemm_tc_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return e;
        mu_gemm_tc_kernel<false><<<grid, THREADS, smem, s>>>(mar, mai, mbr, mbi, static_cast<int>(M), I, chunk, group_kb, mu, err);
    }
    return cudaGetLastError();
}

}  // namespace kpm
