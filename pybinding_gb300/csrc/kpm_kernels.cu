// CUDA kernels of the GB300 KPM engine (sm_103a).
//
// The hot path is one step of the Chebyshev recursion over a block of K
// vectors, y <- H~ x - y, as an ELL SpMM with the two moment dot products of the
// diagonal KPM (m2 = |x|^2, m3 = <y|x>) fused into the same pass
// (cppcore/include/compute/kernel_polynomial.hpp:219-323 is the CPU form).
//
// Layout: the matrix is padded ELL, row-major per row ([row][W] indices and
// values, padding = (row, 0)), so one row's entries are one contiguous load
// shared by the lanes that work on that row. A vector block is row-major,
// [row][K] with the K vectors interleaved per row, so gathering x[col] reads
// K contiguous elements: each lane loads 16 bytes (E elements) and LPR lanes
// cover a row. Vector blocks of all batches live side by side
// ([batch][row][K]) and one launch covers every batch and every system of a
// ragged batch through a tile list (rows of one system x one batch).
//
// Moment sums: each thread accumulates the rows it visits for one (system,
// batch) in the vector precision (FP32 for FP32 vectors: at most a few tiles,
// ~8-64 rows per thread), the two row slots of a warp are added once, and from
// there on everything is FP64: the block sums the per-thread partials in FP64
// shared memory and adds one FP64 atomic per (block, vector, sum) into a
// per-step FP64 accumulator. Per-element FP64 work is avoided on purpose:
// GB300's FP64 rate is ~1/300 of its FP32 rate, and the FP32 partials over a
// bounded number of rows do not add measurable error (moments of a 400k-site
// flake agree to 2.30e-7 of the FP64 recursion with 16-row and with 1024-row
// tiles; the error is the FP32 arithmetic of the recursion itself).
#include "kpm_internal.h"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>
#include <type_traits>
#include <cstdint>
#include <cstring>

namespace kpm {
namespace {

constexpr int BLOCK = 256;
constexpr int WARPS = BLOCK / 32;

// Guards the per-kernel launch caches below (shared-memory attributes set, occupancy): engines
// on different host threads launch concurrently.
std::mutex g_launch_cache_mutex;

// VS: matrix values per entry. FP32 recursions store each value of H~ as an
// unevaluated sum hi + lo of two FP32 numbers (hi = fl32(h), lo = fl32(h - hi),
// h computed in FP64). A plain FP32 H~ shifts the spectrum coherently (every
// hopping carries the same relative rounding) and that bias dominates the FP32
// moment error; the pair removes it for one extra FMA per entry.
template<class V> struct Tr;
template<> struct Tr<float> { using R = float; static constexpr bool C = false; static constexpr int VS = 2; };
template<> struct Tr<double> { using R = double; static constexpr bool C = false; static constexpr int VS = 1; };
template<> struct Tr<float2> { using R = float; static constexpr bool C = true; static constexpr int VS = 2; };
template<> struct Tr<double2> { using R = double; static constexpr bool C = true; static constexpr int VS = 1; };

__device__ __forceinline__ float re32(float a) { return a; }
__device__ __forceinline__ float re32(double a) { return static_cast<float>(a); }
__device__ __forceinline__ float re32(float2 a) { return a.x; }
__device__ __forceinline__ float re32(double2 a) { return static_cast<float>(a.x); }
__device__ __forceinline__ float im32(float2 a) { return a.y; }
__device__ __forceinline__ float im32(double2 a) { return static_cast<float>(a.y); }

__device__ __forceinline__ void vzero(float& a) { a = 0.f; }
__device__ __forceinline__ void vzero(double& a) { a = 0.0; }
__device__ __forceinline__ void vzero(float2& a) { a = make_float2(0.f, 0.f); }
__device__ __forceinline__ void vzero(double2& a) { a = make_double2(0.0, 0.0); }

// acc += a * x
__device__ __forceinline__ void vfma(float& acc, float a, float x) { acc = fmaf(a, x, acc); }
__device__ __forceinline__ void vfma(double& acc, double a, double x) { acc = fma(a, x, acc); }
__device__ __forceinline__ void vfma(float2& acc, float2 a, float2 x) {
    acc.x = fmaf(a.x, x.x, acc.x);
    acc.x = fmaf(-a.y, x.y, acc.x);
    acc.y = fmaf(a.x, x.y, acc.y);
    acc.y = fmaf(a.y, x.x, acc.y);
}
__device__ __forceinline__ void vfma(double2& acc, double2 a, double2 x) {
    acc.x = fma(a.x, x.x, acc.x);
    acc.x = fma(-a.y, x.y, acc.x);
    acc.y = fma(a.x, x.y, acc.y);
    acc.y = fma(a.y, x.x, acc.y);
}
// real matrix value times complex vector element (two FMAs)
__device__ __forceinline__ void vfma(float2& acc, float a, float2 x) {
    acc.x = fmaf(a, x.x, acc.x);
    acc.y = fmaf(a, x.y, acc.y);
}
__device__ __forceinline__ void vfma(double2& acc, double a, double2 x) {
    acc.x = fma(a, x.x, acc.x);
    acc.y = fma(a, x.y, acc.y);
}
__device__ __forceinline__ float vadd(float a, float b) { return a + b; }
__device__ __forceinline__ double vadd(double a, double b) { return a + b; }
__device__ __forceinline__ float2 vadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 vadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float vsub(float a, float b) { return a - b; }
__device__ __forceinline__ double vsub(double a, double b) { return a - b; }
__device__ __forceinline__ float2 vsub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 vsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float vhalf(float a) { return 0.5f * a; }
__device__ __forceinline__ double vhalf(double a) { return 0.5 * a; }
__device__ __forceinline__ float2 vhalf(float2 a) { return make_float2(0.5f * a.x, 0.5f * a.y); }
__device__ __forceinline__ double2 vhalf(double2 a) { return make_double2(0.5 * a.x, 0.5 * a.y); }
// |x|^2
__device__ __forceinline__ float vsq(float a) { return a * a; }
__device__ __forceinline__ double vsq(double a) { return a * a; }
__device__ __forceinline__ float vsq(float2 a) { return fmaf(a.x, a.x, a.y * a.y); }
__device__ __forceinline__ double vsq(double2 a) { return fma(a.x, a.x, a.y * a.y); }
// conj(y) * x
__device__ __forceinline__ float vdre(float y, float x) { return y * x; }
__device__ __forceinline__ double vdre(double y, double x) { return y * x; }
__device__ __forceinline__ float vdre(float2 y, float2 x) { return fmaf(y.x, x.x, y.y * x.y); }
__device__ __forceinline__ double vdre(double2 y, double2 x) { return fma(y.x, x.x, y.y * x.y); }
__device__ __forceinline__ float vdim(float, float) { return 0.f; }
__device__ __forceinline__ double vdim(double, double) { return 0.0; }
__device__ __forceinline__ float vdim(float2 y, float2 x) { return fmaf(y.x, x.y, -y.y * x.x); }
__device__ __forceinline__ double vdim(double2 y, double2 x) { return fma(y.x, x.y, -y.y * x.x); }

// E elements of V in one aligned register pack (4, 8 or 16 bytes)
template<class V, int E>
struct alignas(sizeof(V) * E) Pack {
    V v[E];
};
template<int B> struct Raw;
template<> struct Raw<4> { using T = float; };
template<> struct Raw<8> { using T = float2; };
template<> struct Raw<16> { using T = float4; };

template<class P>
__device__ __forceinline__ P ld_ro(P const* p) {  // read-only path (L1 cached): x gathers
    using T = typename Raw<sizeof(P)>::T;
    T t = __ldg(reinterpret_cast<T const*>(p));
    P r;
    memcpy(&r, &t, sizeof(P));
    return r;
}
template<class P>
__device__ __forceinline__ P ld_l2(P const* p) {  // coherent at L2 (bypasses L1): data written in this launch
    using T = typename Raw<sizeof(P)>::T;
    T t = __ldcg(reinterpret_cast<T const*>(p));
    P r;
    memcpy(&r, &t, sizeof(P));
    return r;
}
template<class P>
__device__ __forceinline__ P ld_stream(P const* p) {  // streamed once: y_old
    using T = typename Raw<sizeof(P)>::T;
    T t = __ldcs(reinterpret_cast<T const*>(p));
    P r;
    memcpy(&r, &t, sizeof(P));
    return r;
}
template<class P>
__device__ __forceinline__ void st_stream(P* p, P const& v) {
    using T = typename Raw<sizeof(P)>::T;
    T t;
    memcpy(&t, &v, sizeof(P));
    __stcs(reinterpret_cast<T*>(p), t);
}

// ------------------------------------------------------------------ diagonal step
// One row of y <- H~ x - y for this lane's E vectors. The row's entries are taken
// in chunks of 4 with every load of a chunk issued before its first use, so a row
// costs two dependent memory round trips (indices, then gathers) rather than one
// per entry; x[r] and y_old[r] are issued ahead of the index loads.
// Compensated row sum of H~ x for FP32 (CR): every term h x is added with an error-free
// transformation -- the product split exactly into fl(h x) + e by an FMA, the sum by Knuth's
// TwoSum -- and the lost parts, with the low halves of the matrix values, gather in a second
// FP32 word, so the row sum is rounded once (as if it were computed exactly) before y_old is
// subtracted. Rounding inside the plain FMA chain is what limits the FP32 recursion's moment
// error (measured on a 395k-site flake: 1.4e-6 of max |mu| at 4098 moments with chained FMAs,
// 4.5e-8 with the row sum rounded once).
__device__ __forceinline__ void two_sum_term(float& sum, float& lo, float h, float hl, float x) {
    float const p = __fmul_rn(h, x);
    float const pe = fmaf(h, x, -p);  // h x - fl(h x), exact
    float const s = __fadd_rn(sum, p);
    float const bb = __fsub_rn(s, sum);
    float const err = __fadd_rn(__fsub_rn(sum, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    sum = s;
    lo = fmaf(hl, x, __fadd_rn(lo, __fadd_rn(err, pe)));
}

// Row sum of H~ x compensated by one FMA per term (CR = 1): s1 = fl(s + fl(h x)); when |s| >=
// |fl(h x)| the difference s - s1 is exact (Fast2Sum), and one FMA gives h x + (s - s1) -- the
// product's rounding plus the sum's -- rounded once; it gathers, with the low halves of the
// matrix values, in a second FP32 word. The rounding inside a row sum that cancels, as the rows
// of high Chebyshev vectors do, is large against the result; this removes it. Measured (NumPy
// emulation of these operations, 395k-site flake, 4098 moments): 3.8e-8 of max |mu| per vector,
// the same as with TwoSum (two_sum_term), against 1.4e-6 with chained FMAs and 3.8e-7 with
// exact products but plain sums; 6 FP32 operations per term against 11 for TwoSum.
__device__ __forceinline__ void fma_compensated_term(float& sum, float& lo, float h, float hl, float x) {
    float const p = __fmul_rn(h, x);
    float const s1 = __fadd_rn(sum, p);
    float const c = fmaf(h, x, __fsub_rn(sum, s1));  // (h x - p) + (sum + p - s1), rounded once
    sum = s1;
    lo = fmaf(hl, x, __fadd_rn(lo, c));
}

// The FP32 row arithmetic of the compensated row sums two vectors at a time: sm_100 and later
// issue FP32 add, multiply and FMA on pairs (__fadd2_rn, __fmul2_rn, __ffma2_rn), one
// instruction for two of a lane's E vectors. Each element rounds as its scalar operation does,
// so the results are the same bits. Chained FMAs (CR = 0) stay scalar: paired, they measured
// slower (506 against 430 us per step on a 128^3 cube, 64 vectors), and the 3-4 instructions
// they issue per entry and vector do not limit the step.
// CR: 0 chained FMAs, 1 FMA-compensated (fma_compensated_term), 2 TwoSum (two_sum_term).
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

template<int E, int CR>
__device__ __forceinline__ void row_terms_f32(float (&sum)[E], float (&lo)[E], float h, float hl,
                                              Pack<float, E> const& x) {
    if constexpr (E % 2 != 0 || CR == 0) {
#pragma unroll
        for (int e = 0; e < E; ++e) {
            if constexpr (CR == 2) two_sum_term(sum[e], lo[e], h, hl, x.v[e]);
            else if constexpr (CR == 1) fma_compensated_term(sum[e], lo[e], h, hl, x.v[e]);
            else { sum[e] = fmaf(h, x.v[e], sum[e]); lo[e] = fmaf(hl, x.v[e], lo[e]); }
        }
    } else {
        float2 const h2 = make_float2(h, h);
        float2 const hl2 = make_float2(hl, hl);
#pragma unroll
        for (int k = 0; k < E; k += 2) {
            float2 const xv = make_float2(x.v[k], x.v[k + 1]);
            float2 s = make_float2(sum[k], sum[k + 1]);
            float2 l = make_float2(lo[k], lo[k + 1]);
            if constexpr (CR == 1) {
                float2 const p = __fmul2_rn(h2, xv);
                float2 const s1 = __fadd2_rn(s, p);
                float2 const c = __ffma2_rn(h2, xv, __fadd2_rn(s, neg2(s1)));
                s = s1;
                l = __ffma2_rn(hl2, xv, __fadd2_rn(l, c));
            } else {  // exact product (FMA split) and Knuth's TwoSum of s + p
                float2 const p = __fmul2_rn(h2, xv);
                float2 const pe = __ffma2_rn(h2, xv, neg2(p));  // h x - fl(h x), exact
                float2 const s1 = __fadd2_rn(s, p);
                float2 const bb = __fadd2_rn(s1, neg2(s));
                float2 const err = __fadd2_rn(__fadd2_rn(s, neg2(__fadd2_rn(s1, neg2(bb)))), __fadd2_rn(p, neg2(bb)));
                s = s1;
                l = __ffma2_rn(hl2, xv, __fadd2_rn(l, __fadd2_rn(err, pe)));
            }
            sum[k] = s.x;
            sum[k + 1] = s.y;
            lo[k] = l.x;
            lo[k + 1] = l.y;
        }
    }
}

// y_new = (sum + lo) - y_old (or (sum + lo) / 2 for the first step), and the moment sums
// m2 += x_r^2, m3 += y_new x_r, two vectors at a time (PAIR) or one
template<int E, bool INIT, bool PAIR>
__device__ __forceinline__ void row_finish_f32(float const (&sum)[E], float const (&lo)[E], Pack<float, E> const& yo,
                                               Pack<float, E> const& xr, Pack<float, E>& yn, float (&m2)[E],
                                               float (&m3)[E]) {
    if constexpr (E % 2 != 0 || !PAIR) {
#pragma unroll
        for (int e = 0; e < E; ++e) {
            float const sv = sum[e] + lo[e];
            yn.v[e] = INIT ? 0.5f * sv : sv - yo.v[e];
            m2[e] = fmaf(xr.v[e], xr.v[e], m2[e]);
            m3[e] = fmaf(yn.v[e], xr.v[e], m3[e]);
        }
    } else {
#pragma unroll
        for (int k = 0; k < E; k += 2) {
            float2 const sv = __fadd2_rn(make_float2(sum[k], sum[k + 1]), make_float2(lo[k], lo[k + 1]));
            float2 const y = INIT ? __fmul2_rn(sv, make_float2(0.5f, 0.5f))
                                  : __fadd2_rn(sv, neg2(make_float2(yo.v[k], yo.v[k + 1])));
            yn.v[k] = y.x;
            yn.v[k + 1] = y.y;
            float2 const xv = make_float2(xr.v[k], xr.v[k + 1]);
            float2 const a = __ffma2_rn(xv, xv, make_float2(m2[k], m2[k + 1]));
            float2 const b = __ffma2_rn(y, xv, make_float2(m3[k], m3[k + 1]));
            m2[k] = a.x;
            m2[k + 1] = a.y;
            m3[k] = b.x;
            m3[k + 1] = b.y;
        }
    }
}

template<class V, int E, int LPR, bool INIT, int U, bool XCOH = false, class MV = V, int CR = 0>
__device__ __forceinline__ void diag_rows(int32_t const* __restrict__ col, MV const* __restrict__ val, int W,
                                          V const* __restrict__ x, V* __restrict__ y, int const (&rr)[U],
                                          bool const (&live)[U], int lane, typename Tr<V>::R (&m2)[E],
                                          typename Tr<V>::R (&m3r)[E], typename Tr<V>::R (&m3i)[E]) {
    constexpr bool CPLX = Tr<V>::C;
    constexpr int K = E * LPR;
    constexpr int VS = Tr<MV>::VS;
    using P = Pack<V, E>;
    P xr[U], yo[U];
    V sum[U][E], lo[U][E];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        if (!live[u]) continue;
        P const* xp = reinterpret_cast<P const*>(x + static_cast<int64_t>(rr[u]) * K) + lane;
        xr[u] = XCOH ? ld_l2(xp) : ld_ro(xp);
        if (!INIT) {  // XCOH: rows written earlier in the same launch are read through L2 only
            P const* yp = reinterpret_cast<P const*>(y + static_cast<int64_t>(rr[u]) * K) + lane;
            yo[u] = XCOH ? ld_l2(yp) : ld_stream(yp);
        }
#pragma unroll
        for (int e = 0; e < E; ++e) { vzero(sum[u][e]); vzero(lo[u][e]); }
    }
    for (int j0 = 0; j0 < W; j0 += 4) {
        int32_t c[U][4];
        P xv[U][4];
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int q = 0; q < 4; ++q)
                c[u][q] = (live[u] && j0 + q < W) ? __ldg(col + static_cast<int64_t>(rr[u]) * W + j0 + q) : 0;
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (live[u] && j0 + q < W) {
                    P const* xp = reinterpret_cast<P const*>(x + static_cast<int64_t>(c[u][q]) * K) + lane;
                    xv[u][q] = XCOH ? ld_l2(xp) : ld_ro(xp);
                }
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (!(live[u] && j0 + q < W)) continue;
                MV const* vp = val + (static_cast<int64_t>(rr[u]) * W + j0 + q) * VS;
                MV const a = vp[0];
                if constexpr (CR != 0) {
                    static_assert(std::is_same_v<V, float> && std::is_same_v<MV, float>, "compensated rows are FP32");
                    row_terms_f32<E, CR>(sum[u], lo[u], a, vp[1], xv[u][q]);
                } else {
#pragma unroll
                    for (int e = 0; e < E; ++e) vfma(sum[u][e], a, xv[u][q].v[e]);
                    if (VS == 2) {
                        MV const b = vp[1];
#pragma unroll
                        for (int e = 0; e < E; ++e) vfma(lo[u][e], b, xv[u][q].v[e]);
                    }
                }
            }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
        if (!live[u]) continue;
        P yn;
        if constexpr (CR != 0) {
            row_finish_f32<E, INIT, true>(sum[u], lo[u], yo[u], xr[u], yn, m2, m3r);
            st_stream(reinterpret_cast<P*>(y + static_cast<int64_t>(rr[u]) * K) + lane, yn);
        } else {
#pragma unroll
            for (int e = 0; e < E; ++e) {
                V const s = (VS == 2) ? vadd(sum[u][e], lo[u][e]) : sum[u][e];
                yn.v[e] = INIT ? vhalf(s) : vsub(s, yo[u].v[e]);
            }
            st_stream(reinterpret_cast<P*>(y + static_cast<int64_t>(rr[u]) * K) + lane, yn);
#pragma unroll
            for (int e = 0; e < E; ++e) {
                m2[e] += vsq(xr[u].v[e]);
                m3r[e] += vdre(yn.v[e], xr[u].v[e]);
                if (CPLX) m3i[e] += vdim(yn.v[e], xr[u].v[e]);
            }
        }
    }
}

// Persistent form: block b takes tiles b, b+G, b+2G, ... so that all blocks sweep the
// rows together in one narrow window (the x rows that neighbouring rows gather stay in
// L2; a contiguous range per block would keep G distant windows alive and re-read x
// from DRAM). Moment partials stay in registers and are reduced over the block and
// added to the FP64 accumulator only when the tile's (system, batch) changes and at
// the end.
template<class V, int E, int LPR>
__device__ __forceinline__ void diag_flush(typename Tr<V>::R (&m2)[E], typename Tr<V>::R (&m3r)[E],
                                           typename Tr<V>::R (&m3i)[E], double* red, double* a) {
    using R = typename Tr<V>::R;
    constexpr bool CPLX = Tr<V>::C;
    constexpr int K = E * LPR;
    constexpr int NV = CPLX ? 3 : 2;
    // the row slots of a warp hold partials of the same vectors: pairwise in the partials'
    // precision (one add for the 32 / LPR = 2 slots of a 16-lane row), then FP64 from here on
#pragma unroll
    for (int off = LPR; off < 32; off <<= 1) {
#pragma unroll
        for (int e = 0; e < E; ++e) {
            m2[e] += __shfl_xor_sync(0xffffffffu, m2[e], off);
            m3r[e] += __shfl_xor_sync(0xffffffffu, m3r[e], off);
            if (CPLX) m3i[e] += __shfl_xor_sync(0xffffffffu, m3i[e], off);
        }
    }
    int const warp = threadIdx.x / 32;
    int const wl = threadIdx.x % 32;
    __syncthreads();  // the previous flush has finished reading `red`
    if (wl < LPR) {
#pragma unroll
        for (int e = 0; e < E; ++e) {
            double* rw = red + (warp * K + wl * E + e) * NV;
            rw[0] = static_cast<double>(m2[e]);
            rw[1] = static_cast<double>(m3r[e]);
            if (CPLX) rw[NV - 1] = static_cast<double>(m3i[e]);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < K * NV; i += BLOCK) {
        double sum = 0.0;
#pragma unroll
        for (int w = 0; w < WARPS; ++w) sum += red[w * K * NV + i];
        atomicAdd(a + i, sum);
    }
#pragma unroll
    for (int e = 0; e < E; ++e) { m2[e] = R(0); m3r[e] = R(0); m3i[e] = R(0); }
}

template<class V, int E, int LPR, bool INIT, int U, class MV, int CR>
__device__ __forceinline__ void diag_step_body(int32_t const* __restrict__ col, MV const* __restrict__ val, int W,
                                               V const* __restrict__ x_all, V* __restrict__ y_all, int64_t batch_stride,
                                               Tile const* __restrict__ tiles, int num_tiles, int32_t row_limit,
                                               int nbatch, double* __restrict__ acc) {
    using R = typename Tr<V>::R;
    constexpr bool CPLX = Tr<V>::C;
    constexpr int K = E * LPR;
    constexpr int RPP = BLOCK / LPR;  // rows per pass of the block
    constexpr int NV = CPLX ? 3 : 2;
    __shared__ double red[WARPS * K * NV];

    int const lane = threadIdx.x % LPR;
    int const slot = threadIdx.x / LPR;
    int const G = gridDim.x;

    R m2[E], m3r[E], m3i[E];
#pragma unroll
    for (int e = 0; e < E; ++e) { m2[e] = R(0); m3r[e] = R(0); m3i[e] = R(0); }
    int cur_sys = -1, cur_batch = -1;

    for (int ti = blockIdx.x; ti < num_tiles; ti += G) {
        Tile const t = tiles[ti];
        if (t.system != cur_sys || t.batch != cur_batch) {
            if (cur_sys >= 0)
                diag_flush<V, E, LPR>(m2, m3r, m3i, red,
                                      acc + static_cast<int64_t>(cur_sys * nbatch + cur_batch) * K * NV);
            cur_sys = t.system;
            cur_batch = t.batch;
        }
        V const* __restrict__ x = x_all + t.batch * batch_stride;
        V* __restrict__ y = y_all + t.batch * batch_stride;
        int const row_end = min(t.row_end, row_limit);
        for (int r = t.row_begin + slot; r < row_end; r += RPP * U) {
            int rr[U];
            bool live[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                rr[u] = r + u * RPP;
                live[u] = rr[u] < row_end;
            }
            diag_rows<V, E, LPR, INIT, U, false, MV, CR>(col, val, W, x, y, rr, live, lane, m2, m3r, m3i);
        }
    }
    if (cur_sys >= 0)
        diag_flush<V, E, LPR>(m2, m3r, m3i, red, acc + static_cast<int64_t>(cur_sys * nbatch + cur_batch) * K * NV);
}

// The FMA-compensated FP32 rows (CR = 1) with every per-vector value held as pairs of vectors
// (float2) from load to store: the paired instructions then need no moves to form their operands,
// and a subtraction is a paired FMA by -1 (same rounding as the scalar subtraction). The same
// bits as fma_compensated_term and the scalar finish.
template<int E, int LPR, bool INIT, int U>
__device__ __forceinline__ void diag_rows_f2(int32_t const* __restrict__ col, float const* __restrict__ val, int W,
                                             float const* __restrict__ x, float* __restrict__ y, int const (&rr)[U],
                                             bool const (&live)[U], int lane, float2 (&m2)[E / 2],
                                             float2 (&m3)[E / 2]) {
    constexpr int K = E * LPR;
    constexpr int H = E / 2;
    using P = Pack<float2, H>;
    float2 const m1 = make_float2(-1.f, -1.f);
    P xr[U], yo[U];
    float2 sum[U][H], lo[U][H];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        if (!live[u]) continue;
        xr[u] = ld_ro(reinterpret_cast<P const*>(x + static_cast<int64_t>(rr[u]) * K) + lane);
        if (!INIT) yo[u] = ld_stream(reinterpret_cast<P const*>(y + static_cast<int64_t>(rr[u]) * K) + lane);
#pragma unroll
        for (int k = 0; k < H; ++k) { sum[u][k] = make_float2(0.f, 0.f); lo[u][k] = make_float2(0.f, 0.f); }
    }
    for (int j0 = 0; j0 < W; j0 += 4) {
        int32_t c[U][4];
        P xv[U][4];
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int q = 0; q < 4; ++q)
                c[u][q] = (live[u] && j0 + q < W) ? __ldg(col + static_cast<int64_t>(rr[u]) * W + j0 + q) : 0;
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (live[u] && j0 + q < W)
                    xv[u][q] = ld_ro(reinterpret_cast<P const*>(x + static_cast<int64_t>(c[u][q]) * K) + lane);
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (!(live[u] && j0 + q < W)) continue;
                float const* vp = val + (static_cast<int64_t>(rr[u]) * W + j0 + q) * 2;
                float2 const h2 = make_float2(vp[0], vp[0]);
                float2 const hl2 = make_float2(vp[1], vp[1]);
#pragma unroll
                for (int k = 0; k < H; ++k) {
                    float2 const xk = xv[u][q].v[k];
                    float2 const p = __fmul2_rn(h2, xk);
                    float2 const s1 = __fadd2_rn(sum[u][k], p);
                    float2 const cc = __ffma2_rn(h2, xk, __ffma2_rn(s1, m1, sum[u][k]));
                    sum[u][k] = s1;
                    lo[u][k] = __ffma2_rn(hl2, xk, __fadd2_rn(lo[u][k], cc));
                }
            }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
        if (!live[u]) continue;
        P yn;
#pragma unroll
        for (int k = 0; k < H; ++k) {
            float2 const sv = __fadd2_rn(sum[u][k], lo[u][k]);
            yn.v[k] = INIT ? __fmul2_rn(sv, make_float2(0.5f, 0.5f)) : __ffma2_rn(yo[u].v[k], m1, sv);
        }
        st_stream(reinterpret_cast<P*>(y + static_cast<int64_t>(rr[u]) * K) + lane, yn);
#pragma unroll
        for (int k = 0; k < H; ++k) {
            m2[k] = __ffma2_rn(xr[u].v[k], xr[u].v[k], m2[k]);
            m3[k] = __ffma2_rn(yn.v[k], xr[u].v[k], m3[k]);
        }
    }
}

template<int E, int LPR, bool INIT, int U>
__device__ __forceinline__ void diag_step_body_f2(int32_t const* __restrict__ col, float const* __restrict__ val,
                                                  int W, float const* __restrict__ x_all, float* __restrict__ y_all,
                                                  int64_t batch_stride, Tile const* __restrict__ tiles, int num_tiles,
                                                  int32_t row_limit, int nbatch, double* __restrict__ acc) {
    constexpr int K = E * LPR;
    constexpr int H = E / 2;
    constexpr int RPP = BLOCK / LPR;
    __shared__ double red[WARPS * K * 2];
    int const lane = threadIdx.x % LPR;
    int const slot = threadIdx.x / LPR;
    int const G = gridDim.x;
    float2 m2p[H], m3p[H];
#pragma unroll
    for (int k = 0; k < H; ++k) { m2p[k] = make_float2(0.f, 0.f); m3p[k] = make_float2(0.f, 0.f); }
    auto flush = [&](int sys, int b) {
        float m2[E], m3r[E], m3i[E];
#pragma unroll
        for (int k = 0; k < H; ++k) {
            m2[2 * k] = m2p[k].x;
            m2[2 * k + 1] = m2p[k].y;
            m3r[2 * k] = m3p[k].x;
            m3r[2 * k + 1] = m3p[k].y;
            m3i[2 * k] = m3i[2 * k + 1] = 0.f;
            m2p[k] = make_float2(0.f, 0.f);
            m3p[k] = make_float2(0.f, 0.f);
        }
        diag_flush<float, E, LPR>(m2, m3r, m3i, red, acc + static_cast<int64_t>(sys * nbatch + b) * K * 2);
    };
    int cur_sys = -1, cur_batch = -1;
    for (int ti = blockIdx.x; ti < num_tiles; ti += G) {
        Tile const t = tiles[ti];
        if (t.system != cur_sys || t.batch != cur_batch) {
            if (cur_sys >= 0) flush(cur_sys, cur_batch);
            cur_sys = t.system;
            cur_batch = t.batch;
        }
        float const* __restrict__ x = x_all + t.batch * batch_stride;
        float* __restrict__ y = y_all + t.batch * batch_stride;
        int const row_end = min(t.row_end, row_limit);
        for (int r = t.row_begin + slot; r < row_end; r += RPP * U) {
            int rr[U];
            bool live[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                rr[u] = r + u * RPP;
                live[u] = rr[u] < row_end;
            }
            diag_rows_f2<E, LPR, INIT, U>(col, val, W, x, y, rr, live, lane, m2p, m3p);
        }
    }
    if (cur_sys >= 0) flush(cur_sys, cur_batch);
}

// Chained FMAs: no register bound (the compiler's own allocation, 64 registers for one row per
// thread). Compensated row sums are held to 4 resident blocks per SM (64 registers; left free,
// the compiler takes 88 and 2 blocks fit).
template<class V, int E, int LPR, bool INIT, int U, class MV = V>
__global__ void __launch_bounds__(BLOCK)
diag_step_kernel(int32_t const* __restrict__ col, MV const* __restrict__ val, int W,
                 V const* __restrict__ x_all, V* __restrict__ y_all, int64_t batch_stride,
                 Tile const* __restrict__ tiles, int num_tiles, int32_t row_limit, int nbatch,
                 double* __restrict__ acc) {
    diag_step_body<V, E, LPR, INIT, U, MV, 0>(col, val, W, x_all, y_all, batch_stride, tiles, num_tiles, row_limit,
                                              nbatch, acc);
}

template<class V, int E, int LPR, bool INIT, int U, class MV, int CR>
__global__ void __launch_bounds__(BLOCK, 4)
diag_step_cr_kernel(int32_t const* __restrict__ col, MV const* __restrict__ val, int W,
                    V const* __restrict__ x_all, V* __restrict__ y_all, int64_t batch_stride,
                    Tile const* __restrict__ tiles, int num_tiles, int32_t row_limit, int nbatch,
                    double* __restrict__ acc) {
    if constexpr (CR == 1 && std::is_same_v<V, float> && std::is_same_v<MV, float> && E % 2 == 0)
        diag_step_body_f2<E, LPR, INIT, U>(col, val, W, x_all, y_all, batch_stride, tiles, num_tiles, row_limit, nbatch,
                                           acc);
    else
        diag_step_body<V, E, LPR, INIT, U, MV, CR>(col, val, W, x_all, y_all, batch_stride, tiles, num_tiles,
                                                   row_limit, nbatch, acc);
}

// ------------------------------------------------------------------ diagonal step, prefetched entries
// The step of diag_step_kernel with the ELL entries copied into shared memory ahead of use.
// Each warp works through chunks of PF_ROWS consecutive rows of a tile (chunks warp,
// warp + WARPS, ... of every tile the block takes) and, while it computes one chunk, the
// column indices and values of its next chunk are in flight as cp.async copies (no registers
// held). A row then costs one memory round trip -- x[r], y_old[r] and every gather issued
// together, the indices coming from shared memory -- instead of two (indices, then gathers),
// and a warp fetches its entries in a few coalesced copies per chunk rather than one small
// dependent load per row. cp.async completion waits are hardware waits on the warp's own
// copies; nothing here waits on another block.
constexpr int PF_ROWS = 16;  // rows per warp chunk (at least one pass of the warp: 32 / LPR rows)
template<int LPR> __host__ __device__ constexpr int pf_rows() { return (32 / LPR) > PF_ROWS ? (32 / LPR) : PF_ROWS; }

__device__ __forceinline__ uint32_t smem_addr(void const* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cp_async4(void* dst, void const* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prior() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// Shared memory of one block: per warp two buffers of one chunk of entries, each buffer
// holding the column indices (padded to 16 bytes) followed by the values.
template<class MV, int LPR>
__host__ __device__ constexpr int pf_col_words(int W) { return ((pf_rows<LPR>() * W + 3) / 4) * 4; }
template<class MV, int LPR>
__host__ __device__ constexpr int pf_buf_words(int W) {
    return pf_col_words<MV, LPR>(W) + pf_rows<LPR>() * W * Tr<MV>::VS * static_cast<int>(sizeof(MV) / 4);
}
template<class MV, int LPR>
size_t pf_smem_bytes(int W) { return static_cast<size_t>(WARPS) * 2 * pf_buf_words<MV, LPR>(W) * 4; }
constexpr size_t PF_SMEM_MAX = 160 * 1024;  // wider rows use the per-row-load step

template<class V, int E, int LPR, bool INIT, int MINB, class MV = V, int RS = 0>
__global__ void __launch_bounds__(BLOCK, MINB)
diag_pf_kernel(int32_t const* __restrict__ col, MV const* __restrict__ val, int W,
               V const* __restrict__ x_all, V* __restrict__ y_all, int64_t batch_stride,
               Tile const* __restrict__ tiles, int num_tiles, int32_t row_limit, int nbatch,
               double* __restrict__ acc) {
    using R = typename Tr<V>::R;
    using P = Pack<V, E>;
    constexpr bool CPLX = Tr<V>::C;
    constexpr int K = E * LPR;
    constexpr int RPW = 32 / LPR;  // rows of a warp per pass
    constexpr int NV = CPLX ? 3 : 2;
    constexpr int VS = Tr<MV>::VS;
    constexpr int MW = static_cast<int>(sizeof(MV) / 4);  // 4-byte words per matrix value
    constexpr int CR = pf_rows<LPR>();                     // rows per warp chunk
    __shared__ double red[WARPS * K * NV];
    extern __shared__ __align__(16) uint32_t pf_words[];

    int const warp = threadIdx.x / 32;
    int const wl = threadIdx.x % 32;
    int const lane = wl % LPR;
    int const sub = wl / LPR;
    int const G = gridDim.x;
    int const col_words = pf_col_words<MV, LPR>(W);
    int const buf_words = pf_buf_words<MV, LPR>(W);
    uint32_t* const wbuf = pf_words + static_cast<size_t>(warp) * 2 * buf_words;

    // the warp's next chunk at or after (ti, c): skips tiles without a chunk for this warp
    auto next_chunk = [&](int& ti, int& c) {
        while (ti < num_tiles) {
            Tile const t = tiles[ti];
            if (t.row_begin + c * CR < min(t.row_end, row_limit)) return;
            ti += G;
            c = warp;
        }
    };
    // copies of the entries of chunk (ti, c) into buffer b
    auto issue = [&](int ti, int c, int b) {
        Tile const t = tiles[ti];
        int const cb = t.row_begin + c * CR;
        int const ce = min(cb + CR, min(t.row_end, row_limit));
        int const ncol = (ce - cb) * W;
        uint32_t* const dst = wbuf + b * buf_words;
        int32_t const* src_c = col + static_cast<int64_t>(cb) * W;
        for (int i = wl; i < ncol; i += 32) cp_async4(dst + i, src_c + i);
        uint32_t const* src_v = reinterpret_cast<uint32_t const*>(val + static_cast<int64_t>(cb) * W * VS);
        int const nval = ncol * VS * MW;
        for (int i = wl; i < nval; i += 32) cp_async4(dst + col_words + i, src_v + i);
    };

    R m2[E], m3r[E], m3i[E];
#pragma unroll
    for (int e = 0; e < E; ++e) { m2[e] = R(0); m3r[e] = R(0); m3i[e] = R(0); }
    int cur_sys = -1, cur_batch = -1;

    int pti = blockIdx.x, pc = warp;  // the chunk whose entries are in flight or landed
    next_chunk(pti, pc);
    if (pti < num_tiles) issue(pti, pc, 0);
    cp_async_commit();
    int buf = 0;

    for (int ti = blockIdx.x; ti < num_tiles; ti += G) {
        Tile const t = tiles[ti];
        if (t.system != cur_sys || t.batch != cur_batch) {
            if (cur_sys >= 0)
                diag_flush<V, E, LPR>(m2, m3r, m3i, red,
                                      acc + static_cast<int64_t>(cur_sys * nbatch + cur_batch) * K * NV);
            cur_sys = t.system;
            cur_batch = t.batch;
        }
        V const* __restrict__ x = x_all + t.batch * batch_stride;
        V* __restrict__ y = y_all + t.batch * batch_stride;
        int const row_end = min(t.row_end, row_limit);
        for (int c = warp; t.row_begin + c * CR < row_end; c += WARPS) {
            // (ti, c) is the chunk (pti, pc) prefetched last: start the copies of the next one
            int nti = pti, nc = pc + WARPS;
            next_chunk(nti, nc);
            if (nti < num_tiles) issue(nti, nc, buf ^ 1);
            cp_async_commit();
            cp_async_wait_prior();  // every group but the newest is complete: this chunk's entries
            __syncwarp();
            int32_t const* const scol = reinterpret_cast<int32_t const*>(wbuf + buf * buf_words);
            MV const* const sval = reinterpret_cast<MV const*>(wbuf + buf * buf_words + col_words);
            int const cb = t.row_begin + c * CR;
            int const ce = min(cb + CR, row_end);
#pragma unroll 1
            for (int lr0 = 0; lr0 < CR; lr0 += RPW) {
                int const lr = lr0 + sub;
                int const r = cb + lr;
                if (r >= ce) continue;
                P const* xp = reinterpret_cast<P const*>(x + static_cast<int64_t>(r) * K) + lane;
                P const xr = ld_ro(xp);
                P yo;
                if (!INIT) yo = ld_stream(reinterpret_cast<P const*>(y + static_cast<int64_t>(r) * K) + lane);
                V sum[E], lo[E];
#pragma unroll
                for (int e = 0; e < E; ++e) { vzero(sum[e]); vzero(lo[e]); }
                int32_t const* crow = scol + lr * W;
                MV const* vrow = sval + lr * W * VS;
                for (int j0 = 0; j0 < W; j0 += 4) {
                    P xv[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        if (j0 + q < W)
                            xv[q] = ld_ro(reinterpret_cast<P const*>(x + static_cast<int64_t>(crow[j0 + q]) * K) + lane);
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        if (j0 + q >= W) continue;
                        MV const a = vrow[(j0 + q) * VS];
                        if constexpr (RS != 0) {
                            row_terms_f32<E, RS>(sum, lo, a, vrow[(j0 + q) * VS + 1], xv[q]);
                        } else {
#pragma unroll
                            for (int e = 0; e < E; ++e) vfma(sum[e], a, xv[q].v[e]);
                            if (VS == 2) {
                                MV const bl = vrow[(j0 + q) * VS + 1];
#pragma unroll
                                for (int e = 0; e < E; ++e) vfma(lo[e], bl, xv[q].v[e]);
                            }
                        }
                    }
                }
                P yn;
                if constexpr (RS != 0) {
                    row_finish_f32<E, INIT, true>(sum, lo, yo, xr, yn, m2, m3r);
                    st_stream(reinterpret_cast<P*>(y + static_cast<int64_t>(r) * K) + lane, yn);
                } else {
#pragma unroll
                    for (int e = 0; e < E; ++e) {
                        V const sv = (VS == 2) ? vadd(sum[e], lo[e]) : sum[e];
                        yn.v[e] = INIT ? vhalf(sv) : vsub(sv, yo.v[e]);
                    }
                    st_stream(reinterpret_cast<P*>(y + static_cast<int64_t>(r) * K) + lane, yn);
#pragma unroll
                    for (int e = 0; e < E; ++e) {
                        m2[e] += vsq(xr.v[e]);
                        m3r[e] += vdre(yn.v[e], xr.v[e]);
                        if (CPLX) m3i[e] += vdim(yn.v[e], xr.v[e]);
                    }
                }
            }
            __syncwarp();  // the buffer is refilled two chunks later
            pti = nti;
            pc = nc;
            buf ^= 1;
        }
    }
    cp_async_commit();
    asm volatile("cp.async.wait_group 0;" ::: "memory");  // nothing may land after the block exits
    if (cur_sys >= 0)
        diag_flush<V, E, LPR>(m2, m3r, m3i, red, acc + static_cast<int64_t>(cur_sys * nbatch + cur_batch) * K * NV);
}

// ------------------------------------------------------------------ off-diagonal step
template<class V, int E, int LPR, bool INIT>
__global__ void __launch_bounds__(BLOCK)
off_step_kernel(int32_t const* __restrict__ col, V const* __restrict__ val, int W,
                V const* __restrict__ x_all, V* __restrict__ y_all, int64_t batch_stride,
                Tile const* __restrict__ tiles, int32_t row_limit, V const* __restrict__ gamma,
                double* __restrict__ acc) {
    using R = typename Tr<V>::R;
    constexpr int K = E * LPR;
    constexpr int RPP = BLOCK / LPR;
    using P = Pack<V, E>;
    Tile const t = tiles[blockIdx.x];
    int const lane = threadIdx.x % LPR;
    int const slot = threadIdx.x / LPR;
    V const* __restrict__ x = x_all + t.batch * batch_stride;
    V* __restrict__ y = y_all + t.batch * batch_stride;
    int const row_end = min(t.row_end, row_limit);
    R dre[E], dim[E];
#pragma unroll
    for (int e = 0; e < E; ++e) { dre[e] = R(0); dim[e] = R(0); }
    constexpr int VS = Tr<V>::VS;
    for (int r = t.row_begin + slot; r < row_end; r += RPP) {
        V sum[E];
#pragma unroll
        for (int e = 0; e < E; ++e) vzero(sum[e]);
        int32_t const* cp = col + static_cast<int64_t>(r) * W;
        V const* vp = val + static_cast<int64_t>(r) * W * VS;
        for (int j = 0; j < W; ++j) {
            int32_t const c = __ldg(cp + j);
            P const xv = ld_ro(reinterpret_cast<P const*>(x + static_cast<int64_t>(c) * K) + lane);
#pragma unroll
            for (int v = 0; v < VS; ++v) {
                V const a = vp[j * VS + v];
#pragma unroll
                for (int e = 0; e < E; ++e) vfma(sum[e], a, xv.v[e]);
            }
        }
        P* yp = reinterpret_cast<P*>(y + static_cast<int64_t>(r) * K) + lane;
        P yn;
        if (INIT) {
#pragma unroll
            for (int e = 0; e < E; ++e) yn.v[e] = vhalf(sum[e]);
        } else {
            P const yo = *yp;
#pragma unroll
            for (int e = 0; e < E; ++e) yn.v[e] = vsub(sum[e], yo.v[e]);
        }
        *yp = yn;
        if (gamma != nullptr) {
            V const g = gamma[r];
#pragma unroll
            for (int e = 0; e < E; ++e) {
                dre[e] += vdre(g, yn.v[e]);
                dim[e] += vdim(g, yn.v[e]);
            }
        }
    }
    if (gamma == nullptr) return;
#pragma unroll
    for (int off = LPR; off < 32; off <<= 1)
#pragma unroll
        for (int e = 0; e < E; ++e) {
            dre[e] += __shfl_xor_sync(0xffffffffu, dre[e], off);
            dim[e] += __shfl_xor_sync(0xffffffffu, dim[e], off);
        }
    __shared__ R red[WARPS][K][2];
    int const warp = threadIdx.x / 32;
    int const wl = threadIdx.x % 32;
    if (wl < LPR)
#pragma unroll
        for (int e = 0; e < E; ++e) {
            red[warp][wl * E + e][0] = dre[e];
            red[warp][wl * E + e][1] = dim[e];
        }
    __syncthreads();
    double* a = acc + static_cast<int64_t>(t.batch) * K * 2;
    for (int i = threadIdx.x; i < K * 2; i += BLOCK) {
        R s = R(0);
#pragma unroll
        for (int w = 0; w < WARPS; ++w) s += red[w][i / 2][i % 2];
        atomicAdd(a + i, static_cast<double>(s));
    }
}

// ------------------------------------------------------------------ dense collection step
int persistent_grid(void const* fn, int num_tiles, size_t smem = 0);

// One row of y <- H~ x - y (or H~ x / 2) for this lane's E vectors and the collected vector
// of the row: x[r] (left side) or V x at row r (right side, V = val2 on the pattern of H~).
// The row's entries go in chunks of 4 with all index loads, then all gathers, issued before
// the first use (as in the diagonal step), so a row costs two dependent round trips.
template<class V, int E, int LPR, bool INIT>
__device__ __forceinline__ void dense_row(int32_t const* __restrict__ col, V const* __restrict__ val,
                                          V const* __restrict__ val2, int W, V const* __restrict__ x,
                                          V* __restrict__ y, int r, int lane, Pack<V, E>& z) {
    constexpr int K = E * LPR;
    constexpr int VS = Tr<V>::VS;
    using P = Pack<V, E>;
    P const* xr_p = reinterpret_cast<P const*>(x + static_cast<int64_t>(r) * K) + lane;
    P yo;
    if (!INIT) yo = ld_stream(reinterpret_cast<P const*>(y + static_cast<int64_t>(r) * K) + lane);
    if (val2 == nullptr) z = ld_ro(xr_p);
    V sum[E], lo[E], sv[E], svl[E];
#pragma unroll
    for (int e = 0; e < E; ++e) { vzero(sum[e]); vzero(lo[e]); vzero(sv[e]); vzero(svl[e]); }
    for (int j0 = 0; j0 < W; j0 += 4) {
        int32_t c[4];
        P xv[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) c[q] = j0 + q < W ? __ldg(col + static_cast<int64_t>(r) * W + j0 + q) : 0;
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (j0 + q < W) xv[q] = ld_ro(reinterpret_cast<P const*>(x + static_cast<int64_t>(c[q]) * K) + lane);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (j0 + q >= W) continue;
            int64_t const vi = (static_cast<int64_t>(r) * W + j0 + q) * VS;
            V const a = val[vi];
#pragma unroll
            for (int e = 0; e < E; ++e) vfma(sum[e], a, xv[q].v[e]);
            if (VS == 2) {
                V const b = val[vi + 1];
#pragma unroll
                for (int e = 0; e < E; ++e) vfma(lo[e], b, xv[q].v[e]);
            }
            if (val2 != nullptr) {
                V const a2 = val2[vi];
#pragma unroll
                for (int e = 0; e < E; ++e) vfma(sv[e], a2, xv[q].v[e]);
                if (VS == 2) {
                    V const b2 = val2[vi + 1];
#pragma unroll
                    for (int e = 0; e < E; ++e) vfma(svl[e], b2, xv[q].v[e]);
                }
            }
        }
    }
    P yn;
#pragma unroll
    for (int e = 0; e < E; ++e) {
        V const s = (VS == 2) ? vadd(sum[e], lo[e]) : sum[e];
        yn.v[e] = INIT ? vhalf(s) : vsub(s, yo.v[e]);
        if (val2 != nullptr) z.v[e] = (VS == 2) ? vadd(sv[e], svl[e]) : sv[e];
    }
    st_stream(reinterpret_cast<P*>(y + static_cast<int64_t>(r) * K) + lane, yn);
}

// Dense-collection step, persistent over interleaved tiles. The collected vector goes to z
// (vector type, [rows][K]) or, for the tensor-core moments GEMM, to FP32 planes zre / zim.
template<class V, int E, int LPR, bool INIT>
__global__ void __launch_bounds__(BLOCK)
dense_step_kernel(int32_t const* __restrict__ col, V const* __restrict__ val, V const* __restrict__ val2, int W,
                  V const* __restrict__ x, V* __restrict__ y, V* __restrict__ z, float* __restrict__ zre,
                  float* __restrict__ zim, Tile const* __restrict__ tiles, int num_tiles) {
    constexpr int K = E * LPR;
    constexpr int RPP = BLOCK / LPR;
    using P = Pack<V, E>;
    int const lane = threadIdx.x % LPR;
    int const slot = threadIdx.x / LPR;
    for (int ti = blockIdx.x; ti < num_tiles; ti += gridDim.x) {
        Tile const t = tiles[ti];
        for (int r = t.row_begin + slot; r < t.row_end; r += RPP) {
            P zv;
            dense_row<V, E, LPR, INIT>(col, val, val2, W, x, y, r, lane, zv);
            int64_t const off = static_cast<int64_t>(r) * K;
            if (zre != nullptr) {
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    __stcs(zre + off + lane * E + e, re32(zv.v[e]));
                    if constexpr (Tr<V>::C) __stcs(zim + off + lane * E + e, im32(zv.v[e]));
                }
            } else {
                st_stream(reinterpret_cast<P*>(z + off) + lane, zv);
            }
        }
    }
}

template<class V, int E, int LPR>
cudaError_t dense_launch(DenseStep const& a, cudaStream_t s) {
    if (a.num_tiles == 0) return cudaSuccess;
    auto const* val = static_cast<V const*>(a.val);
    auto const* val2 = static_cast<V const*>(a.val2);
    auto const* x = static_cast<V const*>(a.x);
    auto* y = static_cast<V*>(a.y);
    auto* z = static_cast<V*>(a.zv != nullptr ? a.zv : a.zx);
    if (a.zre == nullptr && z == nullptr) return cudaErrorInvalidValue;
    if ((a.zv != nullptr) != (a.val2 != nullptr) && a.zre == nullptr) return cudaErrorInvalidValue;
    auto fn = a.init ? dense_step_kernel<V, E, LPR, true> : dense_step_kernel<V, E, LPR, false>;
    int const g = persistent_grid(reinterpret_cast<void const*>(fn), a.num_tiles);
    fn<<<g, BLOCK, 0, s>>>(a.col, val, val2, a.W, x, y, z, a.zre, a.zim, a.tiles, a.num_tiles);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ adjoint step (real types)
// out = S x - yprev (or S x / 2 when half) + a0 v0 + am vm + ap vp   (out and yprev may alias;
// yprev, v0, vm, vp nullable), and when gt is set, per row r and ELL slot j
//   gt[r][j] += sum over the K vectors of x[col_j] * g[r]
// (the gradient of the recursion with respect to the transposed entry S[col_j][r]; the
// pattern of S is symmetric) and gd[r] += sum_k x[r][k] * g[r][k] (the diagonal, also where
// S stores none). The per-step sum over the K vectors of a row is taken in the vectors'
// precision; gt and gd accumulate those over the steps in FP64 for FP64 vectors and, for FP32
// ones, as an unevaluated pair (hi, lo) of FP32 values added to with Knuth's TwoSum (about 48
// bits, no FP64 instruction; a plain FP32 running sum over M/2 steps of terms of both signs lost
// ~1e-4 of the largest gradient). The row loop is uniform over the block so that the lanes of a
// row can reduce with warp shuffles.
template<class V> struct GradSum { using T = double; };
template<> struct GradSum<float> { using T = float2; };
__device__ __forceinline__ double grad_add(double a, double p) { return a + p; }
__device__ __forceinline__ float2 grad_add(float2 a, float p) {
    float const s = __fadd_rn(a.x, p);
    float const bb = __fsub_rn(s, a.x);
    float const e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    return make_float2(s, __fadd_rn(a.y, e));
}

template<class V, int E, int LPR>
__global__ void __launch_bounds__(BLOCK)
adj_step_kernel(int32_t const* __restrict__ col, V const* __restrict__ val, int W, V const* __restrict__ x,
                V const* yprev, V* out, int half, V const* __restrict__ v0, V const* __restrict__ vm,
                V const* __restrict__ vp, V a0, V am, V ap, V const* __restrict__ g,
                typename GradSum<V>::T* __restrict__ gt, typename GradSum<V>::T* __restrict__ gd,
                Tile const* __restrict__ tiles, int num_tiles) {
    static_assert(!Tr<V>::C, "the adjoint step is real");
    using G = typename GradSum<V>::T;
    constexpr int K = E * LPR;
    constexpr int RPP = BLOCK / LPR;
    constexpr int VS = Tr<V>::VS;
    using P = Pack<V, E>;
    int const lane = threadIdx.x % LPR;
    int const slot = threadIdx.x / LPR;
    bool const grad = gt != nullptr;
    // gradient sums (FP64): with fewer entries per row than lanes, lane j owns slot j and lane W
    // the diagonal; their old values are loaded with the row's other loads, so no dependent
    // read-modify-write ends the row
    bool const spread = grad && W < LPR;
    for (int ti = blockIdx.x; ti < num_tiles; ti += gridDim.x) {  // uniform over the block
        Tile const t = tiles[ti];
        for (int rb = t.row_begin; rb < t.row_end; rb += RPP) {
            int const r = rb + slot;
            bool const live = r < t.row_end;
            int const rs = live ? r : t.row_begin;  // dead lanes follow a valid row without storing
            int64_t const off = static_cast<int64_t>(rs) * K;
            P gv, yo, q0;
            G gpre{};
            V gsum = V(0);  // one term per lane and step
            if (spread && live) {
                if (lane < W) gpre = gt[static_cast<int64_t>(r) * W + lane];
                else if (lane == W) gpre = gd[r];
            }
            if (grad) gv = ld_ro(reinterpret_cast<P const*>(g + off) + lane);
            if (out != nullptr && yprev != nullptr) yo = reinterpret_cast<P const*>(yprev + off)[lane];
            if (out != nullptr && v0 != nullptr) q0 = (grad && v0 == g) ? gv : ld_ro(reinterpret_cast<P const*>(v0 + off) + lane);
            if (grad) {
                P const xr = ld_ro(reinterpret_cast<P const*>(x + off) + lane);
                V p = V(0);
#pragma unroll
                for (int e = 0; e < E; ++e) vfma(p, xr.v[e], gv.v[e]);
#pragma unroll
                for (int o = 1; o < LPR; o <<= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
                if (spread) {
                    if (lane == W) gsum += p;
                } else if (live && lane == 0) {
                    gd[r] = grad_add(gd[r], p);
                }
            }
            V sum[E], lo[E];
#pragma unroll
            for (int e = 0; e < E; ++e) { vzero(sum[e]); vzero(lo[e]); }
            for (int j0 = 0; j0 < W; j0 += 4) {
                int32_t c[4];
                P xv[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) c[q] = j0 + q < W ? __ldg(col + static_cast<int64_t>(rs) * W + j0 + q) : 0;
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (j0 + q < W) xv[q] = ld_ro(reinterpret_cast<P const*>(x + static_cast<int64_t>(c[q]) * K) + lane);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if (j0 + q >= W) continue;
                    int64_t const vi = (static_cast<int64_t>(rs) * W + j0 + q) * VS;
                    V const a = val[vi];
#pragma unroll
                    for (int e = 0; e < E; ++e) vfma(sum[e], a, xv[q].v[e]);
                    if (VS == 2) {
                        V const b = val[vi + 1];
#pragma unroll
                        for (int e = 0; e < E; ++e) vfma(lo[e], b, xv[q].v[e]);
                    }
                    if (grad) {
                        V p = V(0);
#pragma unroll
                        for (int e = 0; e < E; ++e) vfma(p, xv[q].v[e], gv.v[e]);
#pragma unroll
                        for (int o = 1; o < LPR; o <<= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
                        if (spread) {
                            if (lane == j0 + q) gsum += p;
                        } else if (live && lane == 0) {
                            gt[static_cast<int64_t>(r) * W + j0 + q] = grad_add(gt[static_cast<int64_t>(r) * W + j0 + q], p);
                        }
                    }
                }
            }
            if (spread && live) {
                if (lane < W) gt[static_cast<int64_t>(r) * W + lane] = grad_add(gpre, gsum);
                else if (lane == W) gd[r] = grad_add(gpre, gsum);
            }
            if (live && out != nullptr) {
                P o;
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    V const sv = (VS == 2) ? vadd(sum[e], lo[e]) : sum[e];
                    o.v[e] = half ? vhalf(sv) : sv;
                    if (yprev != nullptr) o.v[e] -= yo.v[e];
                    if (v0 != nullptr) vfma(o.v[e], a0, q0.v[e]);
                }
                if (vm != nullptr) {
                    P const q = ld_ro(reinterpret_cast<P const*>(vm + off) + lane);
#pragma unroll
                    for (int e = 0; e < E; ++e) vfma(o.v[e], am, q.v[e]);
                }
                if (vp != nullptr) {
                    P const q = ld_ro(reinterpret_cast<P const*>(vp + off) + lane);
#pragma unroll
                    for (int e = 0; e < E; ++e) vfma(o.v[e], ap, q.v[e]);
                }
                reinterpret_cast<P*>(out + off)[lane] = o;
            }
        }
    }
}

template<class V, int E, int LPR>
cudaError_t adj_launch(AdjStep const& a, cudaStream_t s) {
    if (a.num_tiles == 0) return cudaSuccess;
    auto fn = adj_step_kernel<V, E, LPR>;
    int const grid = persistent_grid(reinterpret_cast<void const*>(fn), a.num_tiles);
    fn<<<grid, BLOCK, 0, s>>>(a.col, static_cast<V const*>(a.val), a.W, static_cast<V const*>(a.x),
                              static_cast<V const*>(a.yprev), static_cast<V*>(a.out), a.half ? 1 : 0,
                              static_cast<V const*>(a.v0), static_cast<V const*>(a.vm), static_cast<V const*>(a.vp),
                              static_cast<V>(a.a0), static_cast<V>(a.am), static_cast<V>(a.ap),
                              static_cast<V const*>(a.g), static_cast<typename GradSum<V>::T*>(a.gt),
                              static_cast<typename GradSum<V>::T*>(a.gd), a.tiles, a.num_tiles);
    return cudaGetLastError();
}

template<class V>
__global__ void axpby_kernel(int64_t n, V a, V const* __restrict__ x, V b, V const* __restrict__ y, V* __restrict__ out) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[i] = a * x[i] + (y != nullptr ? b * y[i] : V(0));
}

// ------------------------------------------------------------------ dense combination of stored vectors
// Y[m][i] = sum_n C[m][n] X[n][i] (FP64; C is M x M row-major, X and Y are M rows of I): the
// cotangents of the Kubo-Bastin moments matrix spread onto the stored Chebyshev vectors of the
// other side. A block stages a 32 x 32 tile of C in shared memory and each of its 256 threads
// owns one column i for 32 rows m, so X is read once per 32 rows of Y, coalesced.
constexpr int DC_ROWS = 32;
__global__ void __launch_bounds__(BLOCK)
dense_combine_kernel(double const* __restrict__ C, double const* __restrict__ X, double* __restrict__ Y, int M,
                     int64_t I) {
    __shared__ double sc[DC_ROWS][DC_ROWS + 1];
    int64_t const i = static_cast<int64_t>(blockIdx.x) * BLOCK + threadIdx.x;
    int const m0 = blockIdx.y * DC_ROWS;
    double acc[DC_ROWS];
#pragma unroll
    for (int a = 0; a < DC_ROWS; ++a) acc[a] = 0.0;
    for (int n0 = 0; n0 < M; n0 += DC_ROWS) {
        for (int t = threadIdx.x; t < DC_ROWS * DC_ROWS; t += BLOCK) {
            int const a = t / DC_ROWS, b = t % DC_ROWS;
            sc[a][b] = (m0 + a < M && n0 + b < M) ? C[static_cast<int64_t>(m0 + a) * M + n0 + b] : 0.0;
        }
        __syncthreads();
        int const nb = min(DC_ROWS, M - n0);
        for (int b = 0; b < nb; ++b) {
            double const x = i < I ? X[static_cast<int64_t>(n0 + b) * I + i] : 0.0;
#pragma unroll
            for (int a = 0; a < DC_ROWS; ++a) acc[a] = fma(sc[a][b], x, acc[a]);
        }
        __syncthreads();
    }
    if (i < I)
#pragma unroll
        for (int a = 0; a < DC_ROWS; ++a)
            if (m0 + a < M) Y[static_cast<int64_t>(m0 + a) * I + i] = acc[a];
}

// ------------------------------------------------------------------ FP64 moments-matrix GEMM (split over I)
__device__ __forceinline__ double2 to_cd(float v) { return make_double2(v, 0.0); }
__device__ __forceinline__ double2 to_cd(double v) { return make_double2(v, 0.0); }
__device__ __forceinline__ double2 to_cd(float2 v) { return make_double2(v.x, v.y); }
__device__ __forceinline__ double2 to_cd(double2 v) { return v; }

constexpr int GT = 32;  // output tile and inner chunk

template<class V>
__global__ void __launch_bounds__(BLOCK)
mu_gemm_kernel(V const* __restrict__ A, V const* __restrict__ B, int64_t M, int64_t I, int64_t chunk,
               double* __restrict__ mu) {
    __shared__ double2 As[GT][GT + 1];
    __shared__ double2 Bs[GT][GT + 1];
    int64_t const m0 = blockIdx.x * GT, n0 = blockIdx.y * GT;
    int64_t const i_begin = blockIdx.z * chunk;
    int64_t const i_end = min(I, i_begin + chunk);
    int const tx = threadIdx.x % 16, ty = threadIdx.x / 16;  // 2x2 outputs per thread
    double2 acc[2][2];
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int q = 0; q < 2; ++q) acc[p][q] = make_double2(0.0, 0.0);
    for (int64_t i0 = i_begin; i0 < i_end; i0 += GT) {
        for (int idx = threadIdx.x; idx < GT * GT; idx += BLOCK) {
            int const rr = idx / GT, ii = idx % GT;
            int64_t const gi = i0 + ii;
            As[ii][rr] = (m0 + rr < M && gi < i_end) ? to_cd(A[(m0 + rr) * I + gi]) : make_double2(0.0, 0.0);
            Bs[ii][rr] = (n0 + rr < M && gi < i_end) ? to_cd(B[(n0 + rr) * I + gi]) : make_double2(0.0, 0.0);
        }
        __syncthreads();
#pragma unroll 4
        for (int ii = 0; ii < GT; ++ii) {
#pragma unroll
            for (int p = 0; p < 2; ++p) {
                double2 const a = As[ii][tx + 16 * p];
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    double2 const b = Bs[ii][ty + 16 * q];
                    // a * conj(b)
                    acc[p][q].x = fma(a.x, b.x, fma(a.y, b.y, acc[p][q].x));
                    acc[p][q].y = fma(a.y, b.x, fma(-a.x, b.y, acc[p][q].y));
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            int64_t const m = m0 + tx + 16 * p, n = n0 + ty + 16 * q;
            if (m < M && n < M) {
                atomicAdd(mu + 2 * (n * M + m), acc[p][q].x);
                atomicAdd(mu + 2 * (n * M + m) + 1, acc[p][q].y);
            }
        }
}

// ------------------------------------------------------------------ Kubo-Bastin
__global__ void __launch_bounds__(BLOCK)
kubo_sum_kernel(double const* __restrict__ mu, int64_t M, double const* __restrict__ samples,
                double* __restrict__ sum_nm) {
    extern __shared__ double Tm[];  // M values cos(m theta)
    __shared__ double shr[WARPS], shi[WARPS];
    int const e = blockIdx.x;
    double const en = samples[e];
    double const th = acos(en);
    double const sq = sqrt(1.0 - en * en);
    for (int64_t m = threadIdx.x; m < M; m += BLOCK) Tm[m] = cos(static_cast<double>(m) * th);
    __syncthreads();
    double re = 0.0, im = 0.0;
    int const warp = threadIdx.x / 32, wl = threadIdx.x % 32;
    // sum_n A_n u_n, u_n = sum_m mu(m,n) T_m (column n contiguous in m)
    for (int64_t n = warp; n < M; n += WARPS) {
        double ur = 0.0, ui = 0.0;
        double const* c = mu + 2 * n * M;
        for (int64_t m = wl; m < M; m += 32) {
            ur = fma(c[2 * m], Tm[m], ur);
            ui = fma(c[2 * m + 1], Tm[m], ui);
        }
        for (int off = 16; off > 0; off >>= 1) {
            ur += __shfl_xor_sync(0xffffffffu, ur, off);
            ui += __shfl_xor_sync(0xffffffffu, ui, off);
        }
        if (wl == 0) {
            double const nr = static_cast<double>(n);
            double sn, cn;
            sincos(nr * th, &sn, &cn);
            // A_n = (en - i n sq) (cn + i sn)
            double const ar = en * cn + nr * sq * sn;
            double const ai = en * sn - nr * sq * cn;
            re += ar * ur - ai * ui;
            im += ar * ui + ai * ur;
        }
    }
    // sum_m conj(A_m) v_m, v_m = sum_n mu(m,n) T_n
    for (int64_t m = threadIdx.x; m < M; m += BLOCK) {
        double vr = 0.0, vi = 0.0;
        for (int64_t n = 0; n < M; ++n) {
            vr = fma(mu[2 * (n * M + m)], Tm[n], vr);
            vi = fma(mu[2 * (n * M + m) + 1], Tm[n], vi);
        }
        double const mr = static_cast<double>(m);
        double sm, cm;
        sincos(mr * th, &sm, &cm);
        double const ar = en * cm + mr * sq * sm;
        double const ai = -(en * sm - mr * sq * cm);  // conj(A_m)
        re += ar * vr - ai * vi;
        im += ar * vi + ai * vr;
    }
    for (int off = 16; off > 0; off >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, off);
        im += __shfl_xor_sync(0xffffffffu, im, off);
    }
    if (wl == 0) { shr[warp] = re; shi[warp] = im; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tr = 0.0, ti = 0.0;
        for (int w = 0; w < WARPS; ++w) { tr += shr[w]; ti += shi[w]; }
        double const k = 1.0 / ((1.0 - en * en) * (1.0 - en * en));
        sum_nm[2 * e] = k * tr;
        sum_nm[2 * e + 1] = k * ti;
    }
}

__global__ void kubo_integrate_kernel(double const* __restrict__ sum_nm, double const* __restrict__ samples, int ns,
                                      double const* __restrict__ chem, int nmu, double inv_kbt, double coeff,
                                      double prefix, double* __restrict__ out) {
    int const j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nmu) return;
    double const mu = chem[j];
    double tr = 0.0, ti = 0.0;
    for (int e = 0; e < ns; ++e) {
        // Fermi-Dirac; at T = 0 (inv_kbt infinite) the step function, 1/2 on the edge, where the
        // reference's formula (reconstruct.hpp:126-128) evaluates 0 * inf and returns NaN
        double const fd = isinf(inv_kbt) ? (samples[e] < mu ? 1.0 : (samples[e] > mu ? 0.0 : 0.5))
                                         : 1.0 / (1.0 + exp((samples[e] - mu) * inv_kbt));
        double const w = (e == 0 || e == ns - 1) ? 1.0 : 2.0;
        tr += w * fd * sum_nm[2 * e];
        ti += w * fd * sum_nm[2 * e + 1];
    }
    out[2 * j] = prefix * coeff * tr;
    out[2 * j + 1] = prefix * coeff * ti;
}

int persistent_grid(void const* fn, int num_tiles, size_t smem) {
    constexpr int kMaxDevices = 64;
    static int sms_of[kMaxDevices] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(g_launch_cache_mutex);
    int& sms = sms_of[dev >= 0 && dev < kMaxDevices ? dev : 0];
    if (sms == 0) {
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    // occupancy per kernel, queried once (the recursion launches the same kernels thousands of times)
    static void const* fns[64];
    static size_t smems[64];
    static int occ[64];
    static int nfns = 0;
    int per_sm = 0;
    for (int i = 0; i < nfns; ++i)
        if (fns[i] == fn && smems[i] == smem) per_sm = occ[i];
    if (per_sm == 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, BLOCK, smem) != cudaSuccess || per_sm < 1) {
            cudaGetLastError();
            per_sm = 1;
        }
        if (nfns < 64) { fns[nfns] = fn; smems[nfns] = smem; occ[nfns] = per_sm; ++nfns; }
    }
    return std::max(1, std::min(num_tiles, sms * per_sm));
}

template<class V, int E, int LPR, class MV = V, int CR = 0>
cudaError_t diag_launch_pf(DiagStep const& a, cudaStream_t s) {
    auto const* val = static_cast<MV const*>(a.val);
    auto const* x = static_cast<V const*>(a.x);
    auto* y = static_cast<V*>(a.y);
    size_t const smem = pf_smem_bytes<MV, LPR>(a.W);
    if (smem > PF_SMEM_MAX) return cudaErrorInvalidValue;
    auto run = [&](auto fn) {
        if (smem > 48 * 1024) {
            cudaError_t const e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       static_cast<int>(smem));
            if (e != cudaSuccess) return e;
        }
        int const g = persistent_grid(reinterpret_cast<void const*>(fn), a.num_tiles, smem);
        fn<<<g, BLOCK, smem, s>>>(a.col, val, a.W, x, y, a.batch_stride, a.tiles, a.num_tiles, a.row_limit,
                                  a.nbatch, a.acc);
        return cudaGetLastError();
    };
    // MINB: blocks per SM the register allocation is held to (3, or 4 with a few spilled words
    // of loop state for the FP32 64-vector shape), timed by the autotuner
    if (a.prefetch >= 4) {
        if (a.init) return run(diag_pf_kernel<V, E, LPR, true, 4, MV, CR>);
        return run(diag_pf_kernel<V, E, LPR, false, 4, MV, CR>);
    }
    if (a.init) return run(diag_pf_kernel<V, E, LPR, true, 3, MV, CR>);
    return run(diag_pf_kernel<V, E, LPR, false, 3, MV, CR>);
}

template<class V, int E, int LPR, int U, class MV = V, int CR = 0>
cudaError_t diag_launch_u(DiagStep const& a, cudaStream_t s) {
    auto const* val = static_cast<MV const*>(a.val);
    auto const* x = static_cast<V const*>(a.x);
    auto* y = static_cast<V*>(a.y);
    auto run = [&](auto fn) {
        int const g = persistent_grid(reinterpret_cast<void const*>(fn), a.num_tiles);
        fn<<<g, BLOCK, 0, s>>>(a.col, val, a.W, x, y, a.batch_stride, a.tiles, a.num_tiles, a.row_limit, a.nbatch,
                               a.acc);
        return cudaGetLastError();
    };
    if constexpr (CR == 0) {
        if (a.init) return run(diag_step_kernel<V, E, LPR, true, U, MV>);
        return run(diag_step_kernel<V, E, LPR, false, U, MV>);
    } else {
        if (a.init) return run(diag_step_cr_kernel<V, E, LPR, true, U, MV, CR>);
        return run(diag_step_cr_kernel<V, E, LPR, false, U, MV, CR>);
    }
}


// ------------------------------------------------------------------ two steps per launch
// Phase A of tile t computes T_n on its rows (x = Q = T_{n-1}, y = P = T_{n-2} -> T_n);
// phase B computes T_{n+1} (x = P = T_n, y = Q = T_{n-1} -> T_{n+1}). Phase B of t reads
// T_n on every row its rows touch and overwrites Q rows that phase A of those tiles
// gathers, so it waits until phase A of tiles band[t] = [lo, hi] is done. Work items
// come from a queue in which B_t follows A_hi, dispensed by an atomic counter to blocks
// that start on them at once: a waiting block only waits on phase-A items already being
// processed by running blocks, and phase A never waits. Waits give up after a bounded
// number of polls and raise *error (the host reports a timeout).
__device__ __forceinline__ int ld_acquire(int const* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.s32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

template<class V, int E, int LPR>
__global__ void __launch_bounds__(BLOCK, 4)
diag_pair_kernel(int32_t const* __restrict__ col, V const* __restrict__ val, int W, V* __restrict__ P_all,
                 V* __restrict__ Q_all, int64_t batch_stride, Tile const* __restrict__ tiles,
                 int32_t const* __restrict__ items, int32_t const* __restrict__ band, int num_tiles, int nbatch,
                 int* __restrict__ flags, int seq, unsigned* __restrict__ counter, double* __restrict__ accA,
                 double* __restrict__ accB, int* __restrict__ error, int spin_limit) {
    using R = typename Tr<V>::R;
    constexpr bool CPLX = Tr<V>::C;
    constexpr int K = E * LPR;
    constexpr int RPP = BLOCK / LPR;
    constexpr int NV = CPLX ? 3 : 2;
    __shared__ double red[WARPS * K * NV];
    // per-thread moment partials of both phases live in shared memory (own slot, no sync); only
    // the current item's partials are in registers, which keeps the kernel within 64 registers
    __shared__ R part[2][NV][E][BLOCK];
    __shared__ int s_item[2];
    __shared__ int s_ok;

    int const lane = threadIdx.x % LPR;
    int const slot = threadIdx.x / LPR;
    int const total = 2 * num_tiles;
#pragma unroll
    for (int ph = 0; ph < 2; ++ph)
#pragma unroll
        for (int v = 0; v < NV; ++v)
#pragma unroll
            for (int e = 0; e < E; ++e) part[ph][v][e][threadIdx.x] = R(0);
    // flush the partials of one phase into its FP64 accumulator slot (block-wide)
    auto flush = [&](int ph, double* a) {
        R f2[E], f3r[E], f3i[E];
#pragma unroll
        for (int e = 0; e < E; ++e) {
            f2[e] = part[ph][0][e][threadIdx.x];
            f3r[e] = part[ph][1][e][threadIdx.x];
            f3i[e] = CPLX ? part[ph][NV - 1][e][threadIdx.x] : R(0);
#pragma unroll
            for (int v = 0; v < NV; ++v) part[ph][v][e][threadIdx.x] = R(0);
        }
        diag_flush<V, E, LPR>(f2, f3r, f3i, red, a);
    };
    int curA_sys = -1, curA_b = -1, curB_sys = -1, curB_b = -1;
    for (int iter = 0;; ++iter) {
        int const buf = iter & 1;
        // A ticket is taken only when the block is free to work on it: an item held in
        // reserve by a busy block would delay every B item that waits on it.
        if (threadIdx.x == 0) {
            unsigned const ticket = atomicAdd(counter, 1u);
            s_item[buf] = ticket < static_cast<unsigned>(total) ? items[ticket] : -1;
        }
        __syncthreads();
        int const item = s_item[buf];
        if (item < 0) break;
        int const t = item >> 1;
        int const ph = item & 1;
        Tile const tl = tiles[t];
        V* P = P_all + tl.batch * batch_stride;
        V* Q = Q_all + tl.batch * batch_stride;
        if (ph == 1) {  // phase B waits for phase A of its band
            if (threadIdx.x < 32) {
                int const lo = band[2 * t], hi = band[2 * t + 1];
                bool ok = true;
                for (int u = lo + static_cast<int>(threadIdx.x); u <= hi && ok; u += 32) {
                    int polls = 0;
                    while (ld_acquire(flags + u) < seq) {
                        if (++polls > spin_limit) { ok = false; break; }
                        __nanosleep(64);
                    }
                }
                ok = __all_sync(0xffffffffu, ok);
                if (threadIdx.x == 0) s_ok = ok ? 1 : 0;
            }
            __syncthreads();
            if (!s_ok) {
                if (threadIdx.x == 0) atomicExch(error, 1);
                continue;
            }
        }
        int& cs = ph == 0 ? curA_sys : curB_sys;
        int& cb = ph == 0 ? curA_b : curB_b;
        if (tl.system != cs || tl.batch != cb) {
            if (cs >= 0) flush(ph, (ph == 0 ? accA : accB) + static_cast<int64_t>(cs * nbatch + cb) * K * NV);
            cs = tl.system;
            cb = tl.batch;
        }
        R m2[E], m3r[E], m3i[E];
#pragma unroll
        for (int e = 0; e < E; ++e) { m2[e] = R(0); m3r[e] = R(0); m3i[e] = R(0); }
        if (ph == 0) {  // T_n from Q = T_{n-1} into P = T_{n-2}
            for (int r = tl.row_begin + slot; r < tl.row_end; r += RPP) {
                int rr[1] = {r};
                bool live[1] = {true};
                diag_rows<V, E, LPR, false, 1, false>(col, val, W, Q, P, rr, live, lane, m2, m3r, m3i);
            }
        } else {        // T_{n+1} from P = T_n into Q = T_{n-1}
            for (int r = tl.row_begin + slot; r < tl.row_end; r += RPP) {
                int rr[1] = {r};
                bool live[1] = {true};
                diag_rows<V, E, LPR, false, 1, true>(col, val, W, P, Q, rr, live, lane, m2, m3r, m3i);
            }
        }
#pragma unroll
        for (int e = 0; e < E; ++e) {
            part[ph][0][e][threadIdx.x] += m2[e];
            part[ph][1][e][threadIdx.x] += m3r[e];
            if (CPLX) part[ph][NV - 1][e][threadIdx.x] += m3i[e];
        }
        if (ph == 0) {
            __syncthreads();  // every row of the tile is stored
            if (threadIdx.x == 0) {
                __threadfence();
                st_release(flags + t, seq);
            }
        }
    }
    if (curA_sys >= 0) flush(0, accA + static_cast<int64_t>(curA_sys * nbatch + curA_b) * K * NV);
    if (curB_sys >= 0) flush(1, accB + static_cast<int64_t>(curB_sys * nbatch + curB_b) * K * NV);
}

template<class V, int E, int LPR>
cudaError_t pair_launch(DiagPair const& a, cudaStream_t s) {
    if (a.num_tiles == 0) return cudaSuccess;
    auto fn = diag_pair_kernel<V, E, LPR>;
    int const g = persistent_grid(reinterpret_cast<void const*>(fn), 2 * a.num_tiles);
    fn<<<g, BLOCK, 0, s>>>(a.col, static_cast<V const*>(a.val), a.W, static_cast<V*>(a.P), static_cast<V*>(a.Q),
                           a.batch_stride, a.tiles, a.items, a.band, a.num_tiles, a.nbatch, a.flags, a.seq,
                           a.counter, a.accA, a.accB, a.error, a.spin_limit);
    return cudaGetLastError();
}

template<class V, int E, int LPR>
cudaError_t diag_launch(DiagStep const& a, cudaStream_t s) {
    if (a.num_tiles == 0) return cudaSuccess;
    if (a.real_matrix) {  // complex vectors, real H~ values: two FMAs per entry instead of four
        if constexpr (Tr<V>::C) {
            using MR = typename Tr<V>::R;
            if (a.prefetch) return diag_launch_pf<V, E, LPR, MR>(a, s);
            if (a.unroll == 2) return diag_launch_u<V, E, LPR, 2, MR>(a, s);
            return diag_launch_u<V, E, LPR, 1, MR>(a, s);
        } else {
            return cudaErrorInvalidValue;
        }
    }
    if (a.compensated) {  // FP32 real vectors only
        if constexpr (std::is_same_v<V, float>) {
            if (a.compensated == 2) return diag_launch_u<V, E, LPR, 1, V, 2>(a, s);  // one row per thread
            if (a.prefetch) return diag_launch_pf<V, E, LPR, V, 1>(a, s);
            if (a.unroll == 2) return diag_launch_u<V, E, LPR, 2, V, 1>(a, s);
            return diag_launch_u<V, E, LPR, 1, V, 1>(a, s);
        } else {
            return cudaErrorInvalidValue;
        }
    }
    if (a.prefetch) return diag_launch_pf<V, E, LPR>(a, s);
    if (a.unroll == 2) return diag_launch_u<V, E, LPR, 2>(a, s);
    return diag_launch_u<V, E, LPR, 1>(a, s);
}

template<class V, int E, int LPR>
cudaError_t off_launch(OffStep const& a, cudaStream_t s) {
    if (a.num_tiles == 0) return cudaSuccess;
    auto const* val = static_cast<V const*>(a.val);
    auto const* x = static_cast<V const*>(a.x);
    auto* y = static_cast<V*>(a.y);
    auto const* g = static_cast<V const*>(a.gamma);
    if (a.init)
        off_step_kernel<V, E, LPR, true><<<a.num_tiles, BLOCK, 0, s>>>(a.col, val, a.W, x, y, a.batch_stride,
                                                                       a.tiles, a.row_limit, g, a.acc);
    else
        off_step_kernel<V, E, LPR, false><<<a.num_tiles, BLOCK, 0, s>>>(a.col, val, a.W, x, y, a.batch_stride,
                                                                        a.tiles, a.row_limit, g, a.acc);
    return cudaGetLastError();
}

// supported (E, LPR) shapes per element type: E fills 16 bytes, or E = 1 for one vector
#define KPM_SHAPES_F32(X) X(float, 1, 1) X(float, 4, 2) X(float, 4, 4) X(float, 4, 8) X(float, 4, 16) X(float, 4, 32)
#define KPM_SHAPES_F64(X) X(double, 1, 1) X(double, 2, 2) X(double, 2, 4) X(double, 2, 8) X(double, 2, 16) X(double, 2, 32)
#define KPM_SHAPES_C64(X) X(float2, 1, 1) X(float2, 2, 2) X(float2, 2, 4) X(float2, 2, 8) X(float2, 2, 16) X(float2, 2, 32)
#define KPM_SHAPES_C128(X) X(double2, 1, 1) X(double2, 1, 2) X(double2, 1, 4) X(double2, 1, 8) X(double2, 1, 16) X(double2, 1, 32)

// thinner lane mappings of the same K (half the bytes per lane, twice the lanes per row) for
// the diagonal step: fewer registers per thread, more rows in flight; the autotuner picks
#define KPM_DIAG_ALT_F32(X) X(float, 2, 32) X(float, 2, 16) X(float, 2, 8)
#define KPM_DIAG_ALT_F64(X) X(double, 1, 32) X(double, 1, 16) X(double, 1, 8)
#define KPM_DIAG_ALT_C64(X) X(float2, 1, 32) X(float2, 1, 16) X(float2, 1, 8)

template<class V> constexpr int vcode();
template<> constexpr int vcode<float>() { return V_F32; }
template<> constexpr int vcode<double>() { return V_F64; }
template<> constexpr int vcode<float2>() { return V_C64; }
template<> constexpr int vcode<double2>() { return V_C128; }

// ------------------------------------------------------------------ collect
__global__ void collect_diag_kernel(double const* __restrict__ acc, int NV, int num_systems, int nbatch, int K,
                                    int64_t half_M, int64_t M, int64_t nvec, double* __restrict__ out) {
    int64_t const per_sys = nvec * half_M;
    int64_t const total = per_sys * num_systems;
    int64_t const step_stride = static_cast<int64_t>(num_systems) * nbatch * K * NV;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t const s = i / per_sys;
        int64_t const rem = i % per_sys;
        int64_t const v = rem / half_M;
        int64_t const n = rem % half_M;
        int64_t const b = v / K, j = v % K;
        int64_t const base = ((s * nbatch + b) * K + j) * NV;
        double const m0 = acc[base];
        double const m1r = acc[base + 1];
        double const m1i = NV == 3 ? acc[base + 2] : 0.0;
        double* o = out + ((s * nvec + v) * M) * 2;
        if (n == 0) {
            o[0] = 0.5 * m0; o[1] = 0.0;
            o[2] = m1r; o[3] = m1i;
        } else {
            double const* a = acc + n * step_stride + base;
            double const m2 = a[0], m3r = a[1], m3i = NV == 3 ? a[2] : 0.0;
            o[4 * n] = 2.0 * m2 - m0;  // 2 (m2 - mu0), mu0 = m0 / 2
            o[4 * n + 1] = 0.0;
            o[4 * n + 2] = 2.0 * m3r - m1r;
            o[4 * n + 3] = 2.0 * m3i - m1i;
        }
    }
}

__global__ void average_kernel(double const* __restrict__ per_vec, int num_systems, int64_t nvec, int64_t M,
                               double* __restrict__ out) {
    int64_t const total = static_cast<int64_t>(num_systems) * M;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t const s = i / M, n = i % M;
        double re = 0.0, im = 0.0;
        for (int64_t v = 0; v < nvec; ++v) {
            double const* p = per_vec + ((s * nvec + v) * M + n) * 2;
            re += p[0];
            im += p[1];
        }
        double const inv = nvec != 1 ? 1.0 / static_cast<double>(nvec) : 1.0;
        out[2 * i] = re * inv;
        out[2 * i + 1] = im * inv;
    }
}

// ------------------------------------------------------------------ starters scatter
__device__ __forceinline__ void cvt(float& d, float v) { d = v; }
__device__ __forceinline__ void cvt(double& d, float v) { d = v; }
__device__ __forceinline__ void cvt(float& d, double v) { d = static_cast<float>(v); }
__device__ __forceinline__ void cvt(double& d, double v) { d = v; }
__device__ __forceinline__ void cvt(float2& d, float2 v) { d = v; }
__device__ __forceinline__ void cvt(double2& d, float2 v) { d = make_double2(v.x, v.y); }
__device__ __forceinline__ void cvt(float2& d, double2 v) { d = make_float2(static_cast<float>(v.x), static_cast<float>(v.y)); }
__device__ __forceinline__ void cvt(double2& d, double2 v) { d = v; }

// src in the Hamiltonian's scalar type S, dst in the recursion type V
template<class S, class V>
__global__ void scatter_kernel(S const* __restrict__ src, V* __restrict__ dst, int32_t const* __restrict__ map,
                               int64_t const* __restrict__ sys_off, int num_systems, int64_t nvec, int K,
                               int64_t rows_total) {
    int64_t const v = blockIdx.y;
    for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < rows_total;
         g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int lo = 0, hi = num_systems;  // find s with sys_off[s] <= g < sys_off[s+1]
        while (hi - lo > 1) {
            int const mid = (lo + hi) / 2;
            if (sys_off[mid] <= g) lo = mid; else hi = mid;
        }
        int64_t const off = sys_off[lo];
        int64_t const rows_s = sys_off[lo + 1] - off;
        V value;
        cvt(value, src[off * nvec + v * rows_s + (g - off)]);
        int64_t const b = v / K, j = v % K;
        dst[(b * rows_total + map[g]) * K + j] = value;
    }
}

template<class V>
__global__ void set_units_kernel(V* __restrict__ dst, int32_t const* __restrict__ pos, int64_t nvec, int K,
                                 int64_t rows_total) {
    int64_t const v = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (v >= nvec) return;
    V one;
    vzero(one);
    if constexpr (Tr<V>::C) one.x = 1; else one = 1;
    dst[((v / K) * rows_total + pos[v]) * K + v % K] = one;
}

template<class V>
__global__ void gather_rows_kernel(V const* __restrict__ y, int32_t const* __restrict__ dest, int ndest,
                                   double* __restrict__ out) {
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ndest) return;
    V const v = y[dest[i]];
    if constexpr (Tr<V>::C) {
        out[2 * i] = static_cast<double>(v.x);
        out[2 * i + 1] = static_cast<double>(v.y);
    } else {
        out[2 * i] = static_cast<double>(v);
        out[2 * i + 1] = 0.0;
    }
}

// ------------------------------------------------------------------ Lanczos (FP64)
template<class V>
__device__ __forceinline__ double block_sum(double v, double* sh) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (threadIdx.x % 32 == 0) sh[threadIdx.x / 32] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < WARPS; ++w) s += sh[w];
    return s;
}

template<class V>
__global__ void __launch_bounds__(BLOCK)
lanczos_a_kernel(int32_t const* __restrict__ ip, int32_t const* __restrict__ ix, V const* __restrict__ hv,
                 V const* __restrict__ v1, V* __restrict__ v0, Tile const* __restrict__ tiles,
                 double const* __restrict__ nrm_prev, double* __restrict__ part) {
    __shared__ double sh[WARPS];
    Tile const t = tiles[blockIdx.x];
    double const bp = sqrt(nrm_prev[t.system]);  // beta of the previous iteration (0 at the start)
    double a = 0.0;
    for (int r = t.row_begin + threadIdx.x; r < t.row_end; r += BLOCK) {
        V sum;
        vzero(sum);
        for (int k = ip[r]; k < ip[r + 1]; ++k) vfma(sum, hv[k], v1[ix[k]]);
        V const old = v0[r];
        if constexpr (Tr<V>::C) v0[r] = make_double2(sum.x - bp * old.x, sum.y - bp * old.y);
        else v0[r] = sum - bp * old;
        a += vdre(sum, v1[r]);
    }
    double const s = block_sum<V>(a, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

template<class V>
__global__ void __launch_bounds__(BLOCK)
lanczos_b_kernel(V const* __restrict__ v1, V* __restrict__ v0, Tile const* __restrict__ tiles,
                 double const* __restrict__ alpha, double* __restrict__ part) {
    __shared__ double sh[WARPS];
    Tile const t = tiles[blockIdx.x];
    double const a = alpha[t.system];
    double n2 = 0.0;
    for (int r = t.row_begin + threadIdx.x; r < t.row_end; r += BLOCK) {
        V l = v0[r];
        V const x = v1[r];
        if constexpr (Tr<V>::C) { l.x -= a * x.x; l.y -= a * x.y; }
        else l -= a * x;
        v0[r] = l;
        n2 += vsq(l);
    }
    double const s = block_sum<V>(n2, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// Per-system sums of the per-tile partials of lanczos_a/b in a fixed order (a strided sum
// per thread, then a fixed tree), so that the Lanczos coefficients, and with them the
// spectral bounds, are the same bits on every run: the moments at high n are sensitive to
// the bounds, and two runs must not differ by the order in which blocks finished.
__global__ void __launch_bounds__(BLOCK)
lanczos_reduce_kernel(double const* __restrict__ part, int32_t const* __restrict__ sys_tiles,
                      double* __restrict__ out) {
    __shared__ double sh[WARPS];
    int const s = blockIdx.x;
    double v = 0.0;
    for (int i = sys_tiles[s] + threadIdx.x; i < sys_tiles[s + 1]; i += BLOCK) v += part[i];
    double const tot = block_sum<double>(v, sh);
    if (threadIdx.x == 0) out[s] = tot;
}

template<class V>
__global__ void __launch_bounds__(BLOCK)
lanczos_c_kernel(V* __restrict__ v0, Tile const* __restrict__ tiles, double const* __restrict__ nrm) {
    Tile const t = tiles[blockIdx.x];
    double const inv = 1.0 / sqrt(nrm[t.system]);
    for (int r = t.row_begin + threadIdx.x; r < t.row_end; r += BLOCK) {
        V l = v0[r];
        if constexpr (Tr<V>::C) { l.x *= inv; l.y *= inv; }
        else l *= inv;
        v0[r] = l;
    }
}

// ------------------------------------------------------------------ reconstruction (FP64)
// cos(n t) for the thread's contiguous chunk of n by the Chebyshev recurrence
// T_{n+1} = 2 E T_n - T_{n-1}, seeded with two direct evaluations per chunk.
__global__ void spectral_density_kernel(double const* __restrict__ mu, int64_t M, double const* __restrict__ energy,
                                        int ne, double a, double b, double* __restrict__ out) {
    __shared__ double sh[WARPS];
    int const e = blockIdx.x, c = blockIdx.y;
    double const E = (energy[e] - b) / a;
    double const th = acos(E);
    int64_t const chunk = (M + BLOCK - 1) / BLOCK;
    int64_t const n0 = threadIdx.x * chunk;
    int64_t const n1 = min(M, n0 + chunk);
    double s = 0.0;
    if (n0 < n1) {
        double tm1 = cos(static_cast<double>(n0) * th);
        double t0 = cos(static_cast<double>(n0 + 1) * th);
        double const* m = mu + (static_cast<int64_t>(c) * M) * 2;
        s = m[2 * n0] * tm1;
        for (int64_t n = n0 + 1; n < n1; ++n) {
            s = fma(m[2 * n], t0, s);
            double const tn = fma(2.0 * E, t0, -tm1);
            tm1 = t0;
            t0 = tn;
        }
    }
    double const tot = block_sum<double>(s, sh);
    if (threadIdx.x == 0) {
        double const k = 2.0 / (M_PI * a);
        out[static_cast<int64_t>(c) * ne + e] = k / sqrt(1.0 - E * E) * tot;
    }
}

__global__ void greens_kernel(double const* __restrict__ mu, int64_t M, double const* __restrict__ energy, int ne,
                              double a, double b, double* __restrict__ out) {
    __shared__ double shr[WARPS], shi[WARPS];
    int const e = blockIdx.x, c = blockIdx.y;
    double const E = (energy[e] - b) / a;
    double const th = acos(E);
    int64_t const chunk = (M + BLOCK - 1) / BLOCK;
    int64_t const n0 = threadIdx.x * chunk;
    int64_t const n1 = min(M, n0 + chunk);
    double sr = 0.0, si = 0.0;
    if (n0 < n1) {
        // z_n = exp(-i n t), advanced by w = exp(-i t)
        double zr = cos(static_cast<double>(n0) * th), zi = -sin(static_cast<double>(n0) * th);
        double const wr = cos(th), wi = -sin(th);
        double const* m = mu + (static_cast<int64_t>(c) * M) * 2;
        for (int64_t n = n0; n < n1; ++n) {
            double const mr = m[2 * n], mi = m[2 * n + 1];
            sr += mr * zr - mi * zi;
            si += mr * zi + mi * zr;
            double const nr = zr * wr - zi * wi;
            double const ni = zr * wi + zi * wr;
            zr = nr;
            zi = ni;
        }
    }
    double const tr = block_sum<double>(sr, shr);
    __syncthreads();
    double const ti = block_sum<double>(si, shi);
    if (threadIdx.x == 0) {
        // k = -2i / a / sqrt(1 - E^2); g = k * (tr + i ti)
        double const f = 2.0 / (a * sqrt(1.0 - E * E));
        double* o = out + (static_cast<int64_t>(c) * ne + e) * 2;
        o[0] = f * ti;
        o[1] = -f * tr;
    }
}

int grid_for(int64_t n, int block = BLOCK) {
    int64_t g = (n + block - 1) / block;
    if (g > 152 * 64) g = 152 * 64;
    return static_cast<int>(g < 1 ? 1 : g);
}

}  // namespace

bool diag_shape_supported(int vtype, int E, int LPR) {
#define KPM_CHECK(V, e, l) if (vtype == vcode<V>() && E == e && LPR == l) return true;
    KPM_SHAPES_F32(KPM_CHECK) KPM_SHAPES_F64(KPM_CHECK) KPM_SHAPES_C64(KPM_CHECK) KPM_SHAPES_C128(KPM_CHECK)
#undef KPM_CHECK
    return false;
}

bool diag_pf_supported(int vtype, int W, int LPR) {
    int const cr = std::max(PF_ROWS, 32 / std::max(LPR, 1));
    int const val_words = (vtype == V_C64 || vtype == V_C128) ? 4 : 2;  // per entry (hi/lo pairs for FP32)
    size_t const buf = static_cast<size_t>((cr * W + 3) / 4) * 4 + static_cast<size_t>(cr) * W * val_words;
    return static_cast<size_t>(WARPS) * 2 * buf * 4 <= PF_SMEM_MAX;
}

bool diag_step_supported(int vtype, int E, int LPR) {
#define KPM_CHECK(V, e, l) if (vtype == vcode<V>() && E == e && LPR == l) return true;
    KPM_SHAPES_F32(KPM_CHECK) KPM_SHAPES_F64(KPM_CHECK) KPM_SHAPES_C64(KPM_CHECK) KPM_SHAPES_C128(KPM_CHECK)
    KPM_DIAG_ALT_F32(KPM_CHECK) KPM_DIAG_ALT_F64(KPM_CHECK) KPM_DIAG_ALT_C64(KPM_CHECK)
#undef KPM_CHECK
    return false;
}

cudaError_t launch_diag_pair(DiagPair const& a, cudaStream_t s) {
#define KPM_DISPATCH(V, e, l) if (a.vtype == vcode<V>() && a.E == e && a.LPR == l) return pair_launch<V, e, l>(a, s);
    KPM_SHAPES_F32(KPM_DISPATCH) KPM_SHAPES_F64(KPM_DISPATCH) KPM_SHAPES_C64(KPM_DISPATCH) KPM_SHAPES_C128(KPM_DISPATCH)
#undef KPM_DISPATCH
    return cudaErrorInvalidValue;
}

cudaError_t launch_diag_step(DiagStep const& a, cudaStream_t s) {
#define KPM_DISPATCH(V, e, l) if (a.vtype == vcode<V>() && a.E == e && a.LPR == l) return diag_launch<V, e, l>(a, s);
    KPM_SHAPES_F32(KPM_DISPATCH) KPM_SHAPES_F64(KPM_DISPATCH) KPM_SHAPES_C64(KPM_DISPATCH) KPM_SHAPES_C128(KPM_DISPATCH)
    KPM_DIAG_ALT_F32(KPM_DISPATCH) KPM_DIAG_ALT_F64(KPM_DISPATCH) KPM_DIAG_ALT_C64(KPM_DISPATCH)
#undef KPM_DISPATCH
    return cudaErrorInvalidValue;
}

cudaError_t launch_dense_step(DenseStep const& a, cudaStream_t s) {
#define KPM_DISPATCH(V, e, l) if (a.vtype == vcode<V>() && a.E == e && a.LPR == l) return dense_launch<V, e, l>(a, s);
    KPM_SHAPES_F32(KPM_DISPATCH) KPM_SHAPES_F64(KPM_DISPATCH) KPM_SHAPES_C64(KPM_DISPATCH) KPM_SHAPES_C128(KPM_DISPATCH)
#undef KPM_DISPATCH
    return cudaErrorInvalidValue;
}

cudaError_t launch_mu_gemm_fp64(int vtype, void const* A, void const* B, int64_t M, int64_t I, double* mu,
                                cudaStream_t s) {
    int64_t const tiles = ((M + GT - 1) / GT) * ((M + GT - 1) / GT);
    int64_t splits = std::max<int64_t>(1, (152 * 8 + tiles - 1) / tiles);
    int64_t chunk = (I + splits - 1) / splits;
    chunk = ((chunk + GT - 1) / GT) * GT;
    splits = (I + chunk - 1) / chunk;
    dim3 grid(static_cast<unsigned>((M + GT - 1) / GT), static_cast<unsigned>((M + GT - 1) / GT),
              static_cast<unsigned>(splits));
    switch (vtype) {
        case V_F32: mu_gemm_kernel<float><<<grid, BLOCK, 0, s>>>(static_cast<float const*>(A), static_cast<float const*>(B), M, I, chunk, mu); break;
        case V_F64: mu_gemm_kernel<double><<<grid, BLOCK, 0, s>>>(static_cast<double const*>(A), static_cast<double const*>(B), M, I, chunk, mu); break;
        case V_C64: mu_gemm_kernel<float2><<<grid, BLOCK, 0, s>>>(static_cast<float2 const*>(A), static_cast<float2 const*>(B), M, I, chunk, mu); break;
        default: mu_gemm_kernel<double2><<<grid, BLOCK, 0, s>>>(static_cast<double2 const*>(A), static_cast<double2 const*>(B), M, I, chunk, mu); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_kubo_sum(double const* mu, int64_t M, double const* samples, int ns, double* sum_nm,
                            cudaStream_t s) {
    size_t const smem = sizeof(double) * static_cast<size_t>(M);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kubo_sum_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        if (e != cudaSuccess) return e;
    }
    kubo_sum_kernel<<<ns, BLOCK, smem, s>>>(mu, M, samples, sum_nm);
    return cudaGetLastError();
}

cudaError_t launch_kubo_integrate(double const* sum_nm, double const* samples, int ns, double const* chem, int nmu,
                                  double inv_kbt, double coeff, double prefix, double* out, cudaStream_t s) {
    if (nmu == 0) return cudaSuccess;
    kubo_integrate_kernel<<<(nmu + 127) / 128, 128, 0, s>>>(sum_nm, samples, ns, chem, nmu, inv_kbt, coeff, prefix, out);
    return cudaGetLastError();
}

cudaError_t launch_adj_step(AdjStep const& a, cudaStream_t s) {
#define KPM_DISPATCH(V, e, l) if (a.vtype == vcode<V>() && a.E == e && a.LPR == l) return adj_launch<V, e, l>(a, s);
    KPM_SHAPES_F32(KPM_DISPATCH) KPM_SHAPES_F64(KPM_DISPATCH)
#undef KPM_DISPATCH
    return cudaErrorInvalidValue;
}

cudaError_t launch_axpby(int vtype, int64_t n, double a, void const* x, double b, void const* y, void* out,
                         cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    unsigned const blocks = static_cast<unsigned>(std::min<int64_t>((n + 255) / 256, 152 * 16));
    if (vtype == V_F32)
        axpby_kernel<float><<<blocks, 256, 0, s>>>(n, static_cast<float>(a), static_cast<float const*>(x),
                                                   static_cast<float>(b), static_cast<float const*>(y),
                                                   static_cast<float*>(out));
    else if (vtype == V_F64)
        axpby_kernel<double><<<blocks, 256, 0, s>>>(n, a, static_cast<double const*>(x), b,
                                                    static_cast<double const*>(y), static_cast<double*>(out));
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_dense_combine(double const* C, double const* X, double* Y, int M, int64_t I, cudaStream_t s) {
    if (M <= 0 || I <= 0) return cudaSuccess;
    if ((M + DC_ROWS - 1) / DC_ROWS > 65535) return cudaErrorInvalidValue;
    dim3 const grid(static_cast<unsigned>((I + BLOCK - 1) / BLOCK), static_cast<unsigned>((M + DC_ROWS - 1) / DC_ROWS));
    dense_combine_kernel<<<grid, BLOCK, 0, s>>>(C, X, Y, M, I);
    return cudaGetLastError();
}

cudaError_t launch_off_step(OffStep const& a, cudaStream_t s) {
#define KPM_DISPATCH(V, e, l) if (a.vtype == vcode<V>() && a.E == e && a.LPR == l) return off_launch<V, e, l>(a, s);
    KPM_SHAPES_F32(KPM_DISPATCH) KPM_SHAPES_F64(KPM_DISPATCH) KPM_SHAPES_C64(KPM_DISPATCH) KPM_SHAPES_C128(KPM_DISPATCH)
#undef KPM_DISPATCH
    return cudaErrorInvalidValue;
}

cudaError_t launch_collect_diag(int vtype, double const* acc, int num_systems, int nbatch, int K, int64_t half_M,
                                int64_t M, int64_t nvec, bool average, double* out, cudaStream_t s) {
    int const NV = vtype_nv(vtype);
    (void)average;
    collect_diag_kernel<<<grid_for(static_cast<int64_t>(num_systems) * nvec * half_M), BLOCK, 0, s>>>(
        acc, NV, num_systems, nbatch, K, half_M, M, nvec, out);
    return cudaGetLastError();
}

cudaError_t launch_average(double const* per_vec, int num_systems, int64_t nvec, int64_t M, double* out,
                           cudaStream_t s) {
    average_kernel<<<grid_for(static_cast<int64_t>(num_systems) * M), BLOCK, 0, s>>>(per_vec, num_systems, nvec, M,
                                                                                  out);
    return cudaGetLastError();
}

cudaError_t launch_scatter_starters(int stype, int vtype, void const* src, void* dst, int32_t const* map,
                                    int64_t const* sys_offsets, int num_systems, int64_t nvec, int K, int nbatch,
                                    int64_t rows_total, cudaStream_t s) {
    (void)nbatch;
    if (nvec == 0 || rows_total == 0) return cudaSuccess;
    if (vtype_complex(stype) != vtype_complex(vtype)) return cudaErrorInvalidValue;
    dim3 grid(grid_for(rows_total) > 4096 ? 4096 : grid_for(rows_total), static_cast<unsigned>(nvec));
#define KPM_SC(S, V) scatter_kernel<S, V><<<grid, BLOCK, 0, s>>>(static_cast<S const*>(src), static_cast<V*>(dst), map, sys_offsets, num_systems, nvec, K, rows_total)
    if (stype == V_F32 && vtype == V_F32) KPM_SC(float, float);
    else if (stype == V_F32 && vtype == V_F64) KPM_SC(float, double);
    else if (stype == V_F64 && vtype == V_F32) KPM_SC(double, float);
    else if (stype == V_F64 && vtype == V_F64) KPM_SC(double, double);
    else if (stype == V_C64 && vtype == V_C64) KPM_SC(float2, float2);
    else if (stype == V_C64 && vtype == V_C128) KPM_SC(float2, double2);
    else if (stype == V_C128 && vtype == V_C64) KPM_SC(double2, float2);
    else KPM_SC(double2, double2);
#undef KPM_SC
    return cudaGetLastError();
}

cudaError_t launch_set_units(int vtype, void* dst, int32_t const* pos, int64_t nvec, int K, int64_t rows_total,
                             cudaStream_t s) {
    if (nvec == 0) return cudaSuccess;
    int const g = static_cast<int>((nvec + 127) / 128);
    switch (vtype) {
        case V_F32: set_units_kernel<float><<<g, 128, 0, s>>>(static_cast<float*>(dst), pos, nvec, K, rows_total); break;
        case V_F64: set_units_kernel<double><<<g, 128, 0, s>>>(static_cast<double*>(dst), pos, nvec, K, rows_total); break;
        case V_C64: set_units_kernel<float2><<<g, 128, 0, s>>>(static_cast<float2*>(dst), pos, nvec, K, rows_total); break;
        default: set_units_kernel<double2><<<g, 128, 0, s>>>(static_cast<double2*>(dst), pos, nvec, K, rows_total); break;
    }
    return cudaGetLastError();
}

__global__ void copy_kernel(uint4* __restrict__ dst, uint4 const* __restrict__ src, size_t n16,
                            unsigned char* __restrict__ dtail, unsigned char const* __restrict__ stail, int ntail) {
    size_t const stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n16; i += stride) dst[i] = src[i];
    if (blockIdx.x == 0 && static_cast<int>(threadIdx.x) < ntail) dtail[threadIdx.x] = stail[threadIdx.x];
}

cudaError_t launch_copy(void* dst, void const* src, size_t bytes, cudaStream_t s) {
    if (bytes == 0) return cudaSuccess;
    if ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) % 16 != 0) return cudaErrorInvalidValue;
    size_t const n16 = bytes / 16;
    int const ntail = static_cast<int>(bytes % 16);
    size_t const want = (n16 + 255) / 256;
    int const g = static_cast<int>(want < 1 ? 1 : (want > 152 * 8 ? 152 * 8 : want));
    copy_kernel<<<g, 256, 0, s>>>(static_cast<uint4*>(dst), static_cast<uint4 const*>(src), n16,
                                  static_cast<unsigned char*>(dst) + n16 * 16,
                                  static_cast<unsigned char const*>(src) + n16 * 16, ntail);
    return cudaGetLastError();
}

cudaError_t launch_gather_rows(int vtype, void const* y, int32_t const* dest, int ndest, double* out, cudaStream_t s) {
    if (ndest == 0) return cudaSuccess;
    int const g = (ndest + 127) / 128;
    switch (vtype) {
        case V_F32: gather_rows_kernel<float><<<g, 128, 0, s>>>(static_cast<float const*>(y), dest, ndest, out); break;
        case V_F64: gather_rows_kernel<double><<<g, 128, 0, s>>>(static_cast<double const*>(y), dest, ndest, out); break;
        case V_C64: gather_rows_kernel<float2><<<g, 128, 0, s>>>(static_cast<float2 const*>(y), dest, ndest, out); break;
        default: gather_rows_kernel<double2><<<g, 128, 0, s>>>(static_cast<double2 const*>(y), dest, ndest, out); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_lanczos_a(bool cplx, int32_t const* ip, int32_t const* ix, void const* v, void const* v1, void* v0,
                             Tile const* tiles, int num_tiles, double const* nrm_prev, double* part,
                             int32_t const* sys_tiles, int nsys, double* alpha, cudaStream_t s) {
    if (cplx)
        lanczos_a_kernel<double2><<<num_tiles, BLOCK, 0, s>>>(ip, ix, static_cast<double2 const*>(v),
                                                              static_cast<double2 const*>(v1),
                                                              static_cast<double2*>(v0), tiles, nrm_prev, part);
    else
        lanczos_a_kernel<double><<<num_tiles, BLOCK, 0, s>>>(ip, ix, static_cast<double const*>(v),
                                                             static_cast<double const*>(v1), static_cast<double*>(v0),
                                                             tiles, nrm_prev, part);
    lanczos_reduce_kernel<<<nsys, BLOCK, 0, s>>>(part, sys_tiles, alpha);
    return cudaGetLastError();
}

cudaError_t launch_lanczos_b(bool cplx, void const* v1, void* v0, Tile const* tiles, int num_tiles,
                             double const* alpha, double* part, int32_t const* sys_tiles, int nsys, double* nrm,
                             cudaStream_t s) {
    if (cplx)
        lanczos_b_kernel<double2><<<num_tiles, BLOCK, 0, s>>>(static_cast<double2 const*>(v1),
                                                              static_cast<double2*>(v0), tiles, alpha, part);
    else
        lanczos_b_kernel<double><<<num_tiles, BLOCK, 0, s>>>(static_cast<double const*>(v1), static_cast<double*>(v0),
                                                             tiles, alpha, part);
    lanczos_reduce_kernel<<<nsys, BLOCK, 0, s>>>(part, sys_tiles, nrm);
    return cudaGetLastError();
}

cudaError_t launch_lanczos_c(bool cplx, void* v0, Tile const* tiles, int num_tiles, double const* nrm,
                             cudaStream_t s) {
    if (cplx) lanczos_c_kernel<double2><<<num_tiles, BLOCK, 0, s>>>(static_cast<double2*>(v0), tiles, nrm);
    else lanczos_c_kernel<double><<<num_tiles, BLOCK, 0, s>>>(static_cast<double*>(v0), tiles, nrm);
    return cudaGetLastError();
}

cudaError_t launch_spectral_density(double const* mu, int64_t M, int cols, double const* energy, int ne, double a,
                                    double b, double* out, cudaStream_t s) {
    if (ne == 0 || cols == 0) return cudaSuccess;
    spectral_density_kernel<<<dim3(ne, cols), BLOCK, 0, s>>>(mu, M, energy, ne, a, b, out);
    return cudaGetLastError();
}

cudaError_t launch_greens(double const* mu, int64_t M, int cols, double const* energy, int ne, double a, double b,
                          double* out, cudaStream_t s) {
    if (ne == 0 || cols == 0) return cudaSuccess;
    greens_kernel<<<dim3(ne, cols), BLOCK, 0, s>>>(mu, M, energy, ne, a, b, out);
    return cudaGetLastError();
}

}  // namespace kpm
