// GPU builder of the KPM inputs: honeycomb flakes cut by a polygon and periodic simple
// cubic lattices, as Hamiltonian CSR matrices in pybinding's site order (C ABI in
// kpm_lattice.h).
//
// One thread owns one site or one CSR row and computes everything it needs from the
// lattice's integer structure: its float32 position (the reference's operation order, with
// explicitly rounded adds and multiplies so that nothing is contracted into an FMA), its
// polygon membership, its valid-neighbour count for the dangling-site removal, and the
// sorted entries of its row. Site numbering, hopping numbering and row pointers are
// exclusive prefix sums (a three-pass block scan). No kernel here waits on another block.
#include "kpm_lattice.h"
#include "kpm_gb300.h"
#include "kpm_internal.h"

#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

namespace {

int fail(int code, std::string const& msg) {
    kpm::set_last_error(msg);  // reported by kpm_last_error()
    return code;
}

#define LAT_CUDA(expr)                                                                         \
    do {                                                                                       \
        cudaError_t e_ = (expr);                                                               \
        if (e_ != cudaSuccess) return fail(KPM_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define LAT_CHECK(expr)                \
    do {                               \
        int rc_ = (expr);              \
        if (rc_ != KPM_OK) return rc_; \
    } while (0)

struct Buf {
    void* p = nullptr;
    size_t n = 0;
    Buf() = default;
    Buf(Buf const&) = delete;
    Buf& operator=(Buf const&) = delete;
    ~Buf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t ensure(size_t bytes) {
        if (p && bytes <= n) return cudaSuccess;
        release();
        cudaError_t const e = cudaMalloc(&p, bytes > 0 ? bytes : 16);
        if (e == cudaSuccess) n = bytes;
        return e;
    }
    template<class T> T* as() const { return static_cast<T*>(p); }
};

// Device copy of kpm_honeycomb plus the sites per sublattice.
struct Honey {
    int32_t s0, s1;
    int64_t block;
    float origin[3], a1[3], a2[3], sub[2][3];
    int32_t hop[3][2];
};

constexpr int kThreads = 256;

int grid_for(int64_t n) {
    int64_t const b = (n + kThreads - 1) / kThreads;
    return static_cast<int>(b < 1 ? 1 : (b > 152 * 32 ? 152 * 32 : b));
}

// ------------------------------------------------------------------ exclusive prefix sum
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;

// Exclusive prefix of `v` over the block (blockDim a multiple of 32, at most 1024);
// *total receives the block's sum. Ends with a barrier, so `sh` can be reused.
__device__ int64_t block_exclusive(int64_t v, int64_t* sh, int64_t* total) {
    int const lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int64_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int64_t const y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        int64_t s = lane < nw ? sh[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int64_t const y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) sh[lane] = s;
    }
    __syncthreads();
    int64_t const r = (w > 0 ? sh[w - 1] : 0) + x - v;
    *total = sh[nw - 1];
    __syncthreads();
    return r;
}

__global__ void scan_tiles_kernel(int32_t const* in, int64_t n, int64_t* sums) {
    __shared__ int64_t sh[32];
    int64_t const base = int64_t(blockIdx.x) * kScanTile;
    int64_t s = 0;
    for (int k = 0; k < kScanItems; ++k) {
        int64_t const i = base + k * kScanThreads + threadIdx.x;
        if (i < n) s += in[i];
    }
    int64_t tot;
    block_exclusive(s, sh, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// One block: tile sums -> exclusive tile offsets; sums[nb] = grand total.
__global__ void scan_sums_kernel(int64_t* sums, int64_t nb) {
    __shared__ int64_t sh[32];
    int64_t carry = 0;
    for (int64_t c = 0; c < nb; c += blockDim.x) {
        int64_t const i = c + threadIdx.x;
        int64_t const v = i < nb ? sums[i] : 0;
        int64_t tot;
        int64_t const e = block_exclusive(v, sh, &tot);
        if (i < nb) sums[i] = carry + e;
        carry += tot;
    }
    if (threadIdx.x == 0) sums[nb] = carry;
}

__global__ void scan_apply_kernel(int32_t const* in, int32_t* out, int64_t n, int64_t const* sums) {
    __shared__ int32_t tile[kScanTile];
    __shared__ int64_t sh[32];
    int64_t const base = int64_t(blockIdx.x) * kScanTile;
    for (int k = 0; k < kScanItems; ++k) {
        int64_t const i = base + k * kScanThreads + threadIdx.x;
        tile[k * kScanThreads + threadIdx.x] = i < n ? in[i] : 0;
    }
    __syncthreads();
    int const t0 = threadIdx.x * kScanItems;
    int64_t s = 0;
    for (int k = 0; k < kScanItems; ++k) s += tile[t0 + k];
    int64_t tot;
    int64_t run = sums[blockIdx.x] + block_exclusive(s, sh, &tot);
    for (int k = 0; k < kScanItems; ++k) {  // this thread's own items only
        int32_t const v = tile[t0 + k];
        tile[t0 + k] = static_cast<int32_t>(run);  // the caller rejects totals above INT32_MAX
        run += v;
    }
    __syncthreads();
    for (int k = 0; k < kScanItems; ++k) {
        int64_t const i = base + k * kScanThreads + threadIdx.x;
        if (i < n) out[i] = tile[k * kScanThreads + threadIdx.x];
    }
}

// ------------------------------------------------------------------ honeycomb sites
// Ray casting in float32 as cppcore/src/system/Shape.cpp:54-88: edges whose end points
// have (approximately) equal y are skipped; otherwise the crossing x of the horizontal
// line through the point is compared with the point's x.
__device__ bool polygon_contains(float const* vx, float const* vy, int nv, float px, float py) {
    bool inside = false;
    for (int i = 0, j = nv - 1; i < nv; j = i++) {
        float const x1 = vx[i], x2 = vx[j], y1 = vy[i], y2 = vy[j];
        float const diff = fabsf(__fsub_rn(y1, y2));
        float const scale = fabsf(__fadd_rn(y1, y2));
        if (diff <= __fmul_rn(FLT_EPSILON, scale) || diff <= FLT_MIN) continue;
        float const k = __fdiv_rn(__fsub_rn(x2, x1), __fsub_rn(y2, y1));
        bool const crosses_y = (y1 > py) != (y2 > py);
        float const x_side = __fadd_rn(__fmul_rn(k, __fsub_rn(py, y1)), x1);
        if (crosses_y && px > x_side) inside = !inside;
    }
    return inside;
}

// Foundation index of the h-th neighbour of the site (n, a, b), or -1 outside the
// foundation. A sites reach B sites at +hop[h], B sites reach A sites at -hop[h].
__device__ __forceinline__ int64_t honey_neighbor(Honey const& p, int n, int a, int b, int h) {
    int const sgn = n == 0 ? 1 : -1;
    int const na = a + sgn * p.hop[h][0], nb = b + sgn * p.hop[h][1];
    if (na < 0 || na >= p.s0 || nb < 0 || nb >= p.s1) return -1;
    return (1 - n) * p.block + int64_t(nb) * p.s0 + na;
}

__device__ __forceinline__ void honey_cell(Honey const& p, int64_t f, int& n, int& a, int& b) {
    n = f >= p.block ? 1 : 0;
    int64_t const rem = f - n * p.block;
    b = static_cast<int>(rem / p.s0);
    a = static_cast<int>(rem - int64_t(b) * p.s0);
}

// Foundation positions (Foundation.cpp:25-48): ps = origin + sub[n]; pb = ps (b = 0) or
// ps + b a2; pa = pb + a a1, each in float32.
__global__ void honeycomb_sites_kernel(Honey p, float const* vx, float const* vy, int nv, float* fx, float* fy,
                                       float* fz, int32_t* valid) {
    int64_t const total = 2 * p.block;
    for (int64_t f = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; f < total; f += int64_t(gridDim.x) * blockDim.x) {
        int n, a, b;
        honey_cell(p, f, n, a, b);
        float pos[3];
        for (int c = 0; c < 3; ++c) {
            float const ps = __fadd_rn(p.origin[c], p.sub[n][c]);
            float const pb = b == 0 ? ps : __fadd_rn(ps, __fmul_rn(static_cast<float>(b), p.a2[c]));
            pos[c] = __fadd_rn(pb, __fmul_rn(static_cast<float>(a), p.a1[c]));
        }
        fx[f] = pos[0];
        fy[f] = pos[1];
        fz[f] = pos[2];
        valid[f] = polygon_contains(vx, vy, nv, pos[0], pos[1]) ? 1 : 0;
    }
}

// One pass of the dangling-site removal: a valid site with fewer than `min_nb` valid
// neighbours is removed. Passes run until one removes nothing. Sites are removed in place,
// so a pass may see a neighbour removed earlier in the same pass; removal is monotone and
// a site of the k-core never drops below `min_nb`, so the fixed point is the k-core,
// the same set as the reference's recursive clearing (Foundation.cpp:73-101).
__global__ void honeycomb_kcore_kernel(Honey p, int32_t* valid, int min_nb, int* changed) {
    int64_t const total = 2 * p.block;
    for (int64_t f = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; f < total; f += int64_t(gridDim.x) * blockDim.x) {
        if (__ldcg(valid + f) == 0) continue;
        int n, a, b;
        honey_cell(p, f, n, a, b);
        int cnt = 0;
        for (int h = 0; h < 3; ++h) {
            int64_t const t = honey_neighbor(p, n, a, b, h);
            if (t >= 0 && __ldcg(valid + t) != 0) ++cnt;
        }
        if (cnt < min_nb) {
            valid[f] = 0;
            *changed = 1;
        }
    }
}

__global__ void compact_sites_kernel(int64_t total, int32_t const* valid, int32_t const* fin, float const* fx,
                                     float const* fy, float const* fz, float* x, float* y, float* z, int32_t* flat) {
    for (int64_t f = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; f < total; f += int64_t(gridDim.x) * blockDim.x) {
        if (!valid[f]) continue;
        int32_t const r = fin[f];
        x[r] = fx[f];
        y[r] = fy[f];
        z[r] = fz[f];
        flat[r] = static_cast<int32_t>(f);
    }
}

// bits[h * nsub0 + r] = 1 when A site r has its h-th neighbour.
__global__ void honeycomb_bits_kernel(Honey p, int64_t nsub0, int32_t const* flat, int32_t const* valid,
                                      int32_t* bits) {
    for (int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r < nsub0; r += int64_t(gridDim.x) * blockDim.x) {
        int n, a, b;
        honey_cell(p, flat[r], n, a, b);
        for (int h = 0; h < 3; ++h) {
            int64_t const t = honey_neighbor(p, 0, a, b, h);
            bits[h * nsub0 + r] = (t >= 0 && valid[t]) ? 1 : 0;
        }
    }
}

__global__ void honeycomb_hops_kernel(Honey p, int64_t nsub0, int32_t const* flat, int32_t const* bits,
                                      int32_t const* pos, int32_t const* fin, int32_t* rows, int32_t* cols) {
    for (int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; j < 3 * nsub0; j += int64_t(gridDim.x) * blockDim.x) {
        if (!bits[j]) continue;
        int const h = static_cast<int>(j / nsub0);
        int64_t const r = j - h * nsub0;
        int n, a, b;
        honey_cell(p, flat[r], n, a, b);
        int64_t const t = honey_neighbor(p, 0, a, b, h);
        rows[pos[j]] = static_cast<int32_t>(r);
        cols[pos[j]] = fin[t];
    }
}

// ------------------------------------------------------------------ CSR rows
template<class R, int NC>
struct Val {
    R c[NC];
};

template<class R, int NC>
__device__ __forceinline__ Val<R, NC> load_val(R const* p, int64_t i) {
    Val<R, NC> v;
    for (int k = 0; k < NC; ++k) v.c[k] = p[i * NC + k];
    return v;
}

template<class R, int NC>
__device__ __forceinline__ bool nonzero_at(R const* p, int64_t i) {
    bool nz = false;
    for (int k = 0; k < NC; ++k) nz |= p[i * NC + k] != R(0);
    return nz;
}

template<class R, int NC>
__device__ __forceinline__ Val<R, NC> conj_val(Val<R, NC> v) {
    if (NC == 2) v.c[NC - 1] = -v.c[NC - 1];
    return v;
}

// Sort the m (<= 7) entries of one row by column (columns are distinct) and store them.
template<class R, int NC>
__device__ __forceinline__ void store_row(int32_t* col, Val<R, NC>* val, int m, int64_t at, int32_t* indices,
                                          R* values) {
    for (int i = 1; i < m; ++i)
        for (int j = i; j > 0 && col[j - 1] > col[j]; --j) {
            int32_t const tc = col[j];
            col[j] = col[j - 1];
            col[j - 1] = tc;
            Val<R, NC> const tv = val[j];
            val[j] = val[j - 1];
            val[j - 1] = tv;
        }
    for (int i = 0; i < m; ++i) {
        indices[at + i] = col[i];
        for (int k = 0; k < NC; ++k) values[(at + i) * NC + k] = val[i].c[k];
    }
}

// Row lengths (counts[nsites] stays 0 so that the scan gives all nsites + 1 pointers).
template<class R, int NC>
__global__ void honeycomb_counts_kernel(Honey p, int64_t nsites, int64_t nsub0, int32_t const* flat,
                                        int32_t const* valid, int32_t const* bits, R const* onsite, int32_t* counts) {
    for (int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r < nsites; r += int64_t(gridDim.x) * blockDim.x) {
        int cnt = 0;
        if (r < nsub0) {
            for (int h = 0; h < 3; ++h) cnt += bits[h * nsub0 + r];
        } else {
            int n, a, b;
            honey_cell(p, flat[r], n, a, b);
            for (int h = 0; h < 3; ++h) {
                int64_t const t = honey_neighbor(p, 1, a, b, h);
                if (t >= 0 && valid[t]) ++cnt;
            }
        }
        if (onsite && nonzero_at<R, NC>(onsite, r)) ++cnt;
        counts[r] = cnt;
    }
}

// Row entries (Hamiltonian.hpp:74-100): an A row holds its bonds' values, a B row the
// conjugates of the bonds that reach it, and each row its non-zero onsite energy.
template<class R, int NC>
__global__ void honeycomb_fill_kernel(Honey p, int64_t nsites, int64_t nsub0, int32_t const* flat,
                                      int32_t const* valid, int32_t const* fin, int32_t const* bits,
                                      int32_t const* pos, R const* hopv, Val<R, NC> hop_const, R const* onsite,
                                      int32_t const* indptr, int32_t* indices, R* values) {
    for (int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r < nsites; r += int64_t(gridDim.x) * blockDim.x) {
        int32_t col[4];
        Val<R, NC> val[4];
        int m = 0;
        if (onsite && nonzero_at<R, NC>(onsite, r)) {
            col[m] = static_cast<int32_t>(r);
            val[m] = load_val<R, NC>(onsite, r);
            ++m;
        }
        int n, a, b;
        honey_cell(p, flat[r], n, a, b);
        for (int h = 0; h < 3; ++h) {
            if (r < nsub0) {
                int64_t const j = h * nsub0 + r;
                if (!bits[j]) continue;
                col[m] = fin[honey_neighbor(p, 0, a, b, h)];
                val[m] = hopv ? load_val<R, NC>(hopv, pos[j]) : hop_const;
                ++m;
            } else {
                int64_t const t = honey_neighbor(p, 1, a, b, h);
                if (t < 0 || !valid[t]) continue;
                int32_t const s = fin[t];  // the A site whose h-th bond reaches this row
                col[m] = s;
                val[m] = conj_val<R, NC>(hopv ? load_val<R, NC>(hopv, pos[h * nsub0 + s]) : hop_const);
                ++m;
            }
        }
        store_row<R, NC>(col, val, m, indptr[r], indices, values);
    }
}

// ------------------------------------------------------------------ simple cubic
__device__ __forceinline__ int32_t cubic_neighbor(int32_t L, int64_t i, int d) {
    int32_t const x = static_cast<int32_t>(i % L), y = static_cast<int32_t>((i / L) % L),
                  z = static_cast<int32_t>(i / (int64_t(L) * L));
    int const dx = d == 0 ? 1 : (d == 1 ? -1 : 0);
    int const dy = d == 2 ? 1 : (d == 3 ? -1 : 0);
    int const dz = d == 4 ? 1 : (d == 5 ? -1 : 0);
    int32_t const xn = (x + dx + L) % L, yn = (y + dy + L) % L, zn = (z + dz + L) % L;
    return (zn * L + yn) * L + xn;
}

__global__ void cubic_sites_kernel(int32_t L, int64_t n, float* x, float* y, float* z) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        x[i] = static_cast<float>(i % L);
        y[i] = static_cast<float>((i / L) % L);
        z[i] = static_cast<float>(i / (int64_t(L) * L));
    }
}

__global__ void cubic_hops_kernel(int32_t L, int64_t n, int32_t* rows, int32_t* cols) {
    for (int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; j < 6 * n; j += int64_t(gridDim.x) * blockDim.x) {
        int const d = static_cast<int>(j / n);
        int64_t const i = j - d * n;
        rows[j] = static_cast<int32_t>(i);
        cols[j] = cubic_neighbor(L, i, d);
    }
}

template<class R, int NC>
__global__ void cubic_counts_kernel(int64_t n, R const* onsite, int32_t* counts) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        counts[i] = 6 + ((onsite && nonzero_at<R, NC>(onsite, i)) ? 1 : 0);
}

template<class R, int NC>
__global__ void cubic_fill_kernel(int32_t L, int64_t n, Val<R, NC> hop_const, R const* onsite, int32_t const* indptr,
                                  int32_t* indices, R* values) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        int32_t col[7];
        Val<R, NC> val[7];
        int m = 0;
        for (int d = 0; d < 6; ++d) {
            col[m] = cubic_neighbor(L, i, d);
            val[m] = hop_const;
            ++m;
        }
        if (onsite && nonzero_at<R, NC>(onsite, i)) {
            col[m] = static_cast<int32_t>(i);
            val[m] = load_val<R, NC>(onsite, i);
            ++m;
        }
        store_row<R, NC>(col, val, m, indptr[i], indices, values);
    }
}

// Call f(R{}, std::integral_constant<int, NC>{}) for a dtype of kpm_gb300.h.
template<class F>
int with_dtype(int dtype, F&& f) {
    switch (dtype) {
        case KPM_F32: return f(float{}, std::integral_constant<int, 1>{});
        case KPM_F64: return f(double{}, std::integral_constant<int, 1>{});
        case KPM_C64: return f(float{}, std::integral_constant<int, 2>{});
        case KPM_C128: return f(double{}, std::integral_constant<int, 2>{});
        default: return fail(KPM_ERR_VALUE, "unknown dtype");
    }
}

}  // namespace

// ====================================================================== builder state
struct kpm_lattice {
    enum Kind { HONEYCOMB, CUBIC } kind = HONEYCOMB;
    Honey hp{};
    int32_t L = 0;
    int64_t total = 0, nsites = 0, nsub0 = 0, nhops = 0;
    double build_time = 0, csr_time = 0;
    int64_t launches = 0;  // kernels launched by this builder
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    Buf valid, fin, fx, fy, fz, x, y, z, flat, bits, pos, sums, flag, verts;
    Buf counts, indptr, indices, values, hopv, onsite, rows, cols;

    ~kpm_lattice() {
        if (stream) cudaStreamSynchronize(stream);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }

    int init() {
        LAT_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        LAT_CUDA(cudaEventCreate(&ev0));
        LAT_CUDA(cudaEventCreate(&ev1));
        return KPM_OK;
    }

    // Exclusive prefix sum of n int32 values; *total = their sum (must fit int32).
    int scan(int32_t const* in, int32_t* out, int64_t n, int64_t* sum) {
        *sum = 0;
        if (n == 0) return KPM_OK;
        int64_t const nb = (n + kScanTile - 1) / kScanTile;
        LAT_CUDA(sums.ensure(sizeof(int64_t) * (nb + 1)));
        scan_tiles_kernel<<<static_cast<unsigned>(nb), kScanThreads, 0, stream>>>(in, n, sums.as<int64_t>());
        scan_sums_kernel<<<1, 1024, 0, stream>>>(sums.as<int64_t>(), nb);
        scan_apply_kernel<<<static_cast<unsigned>(nb), kScanThreads, 0, stream>>>(in, out, n, sums.as<int64_t>());
        launches += 3;
        LAT_CUDA(cudaGetLastError());
        LAT_CUDA(cudaMemcpyAsync(sum, sums.as<int64_t>() + nb, sizeof(int64_t), cudaMemcpyDeviceToHost, stream));
        LAT_CUDA(cudaStreamSynchronize(stream));
        if (*sum > INT32_MAX) return fail(KPM_ERR_VALUE, "the lattice exceeds int32 indices");
        return KPM_OK;
    }

    double elapsed() {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, ev0, ev1) != cudaSuccess) return 0;
        return ms * 1e-3;
    }

    int build_honeycomb(float const* vertices, int nv, int min_nb) {
        std::vector<float> hv(2 * static_cast<size_t>(nv));
        for (int i = 0; i < nv; ++i) {
            hv[i] = vertices[2 * i];
            hv[nv + i] = vertices[2 * i + 1];
        }
        LAT_CUDA(cudaEventRecord(ev0, stream));
        LAT_CUDA(verts.ensure(sizeof(float) * hv.size()));
        LAT_CUDA(cudaMemcpyAsync(verts.p, hv.data(), sizeof(float) * hv.size(), cudaMemcpyHostToDevice, stream));
        total = 2 * hp.block;
        LAT_CUDA(valid.ensure(sizeof(int32_t) * total));
        LAT_CUDA(fin.ensure(sizeof(int32_t) * total));
        LAT_CUDA(fx.ensure(sizeof(float) * total));
        LAT_CUDA(fy.ensure(sizeof(float) * total));
        LAT_CUDA(fz.ensure(sizeof(float) * total));
        LAT_CUDA(flag.ensure(sizeof(int)));
        float const* vx = verts.as<float>();
        honeycomb_sites_kernel<<<grid_for(total), kThreads, 0, stream>>>(hp, vx, vx + nv, nv, fx.as<float>(),
                                                                         fy.as<float>(), fz.as<float>(),
                                                                         valid.as<int32_t>());
        ++launches;
        LAT_CUDA(cudaGetLastError());
        if (min_nb > 0) {
            bool settled = false;
            for (int64_t it = 0; it <= total && !settled; ++it) {  // each unsettled pass removes a site
                int changed = 0;
                LAT_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), stream));
                honeycomb_kcore_kernel<<<grid_for(total), kThreads, 0, stream>>>(hp, valid.as<int32_t>(), min_nb,
                                                                                 flag.as<int>());
                ++launches;
                LAT_CUDA(cudaGetLastError());
                LAT_CUDA(cudaMemcpyAsync(&changed, flag.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
                LAT_CUDA(cudaStreamSynchronize(stream));
                settled = changed == 0;
            }
            if (!settled) return fail(KPM_ERR_RUNTIME, "dangling-site removal did not settle");
        }
        LAT_CHECK(scan(valid.as<int32_t>(), fin.as<int32_t>(), total, &nsites));
        int32_t n0 = 0;  // valid sites of sublattice A = exclusive prefix at the first B site
        LAT_CUDA(cudaMemcpyAsync(&n0, fin.as<int32_t>() + hp.block, sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
        LAT_CUDA(cudaStreamSynchronize(stream));
        nsub0 = n0;
        LAT_CUDA(x.ensure(sizeof(float) * nsites));
        LAT_CUDA(y.ensure(sizeof(float) * nsites));
        LAT_CUDA(z.ensure(sizeof(float) * nsites));
        LAT_CUDA(flat.ensure(sizeof(int32_t) * nsites));
        compact_sites_kernel<<<grid_for(total), kThreads, 0, stream>>>(
            total, valid.as<int32_t>(), fin.as<int32_t>(), fx.as<float>(), fy.as<float>(), fz.as<float>(),
            x.as<float>(), y.as<float>(), z.as<float>(), flat.as<int32_t>());
        ++launches;
        LAT_CUDA(cudaGetLastError());
        LAT_CUDA(bits.ensure(sizeof(int32_t) * 3 * nsub0));
        LAT_CUDA(pos.ensure(sizeof(int32_t) * 3 * nsub0));
        if (nsub0 > 0) {
            honeycomb_bits_kernel<<<grid_for(nsub0), kThreads, 0, stream>>>(hp, nsub0, flat.as<int32_t>(),
                                                                            valid.as<int32_t>(), bits.as<int32_t>());
            ++launches;
            LAT_CUDA(cudaGetLastError());
        }
        LAT_CHECK(scan(bits.as<int32_t>(), pos.as<int32_t>(), 3 * nsub0, &nhops));
        LAT_CUDA(cudaEventRecord(ev1, stream));
        LAT_CUDA(cudaStreamSynchronize(stream));
        build_time = elapsed();
        fx.release();  // foundation positions are no longer needed
        fy.release();
        fz.release();
        return KPM_OK;
    }

    int build_cubic() {
        LAT_CUDA(cudaEventRecord(ev0, stream));
        nsites = nsub0 = total = int64_t(L) * L * L;
        nhops = 6 * nsites;
        LAT_CUDA(x.ensure(sizeof(float) * nsites));
        LAT_CUDA(y.ensure(sizeof(float) * nsites));
        LAT_CUDA(z.ensure(sizeof(float) * nsites));
        cubic_sites_kernel<<<grid_for(nsites), kThreads, 0, stream>>>(L, nsites, x.as<float>(), y.as<float>(),
                                                                       z.as<float>());
        ++launches;
        LAT_CUDA(cudaGetLastError());
        LAT_CUDA(cudaEventRecord(ev1, stream));
        LAT_CUDA(cudaStreamSynchronize(stream));
        build_time = elapsed();
        return KPM_OK;
    }

    int hoppings(int32_t* hrows, int32_t* hcols) {
        if (nhops == 0) return KPM_OK;
        LAT_CUDA(rows.ensure(sizeof(int32_t) * nhops));
        LAT_CUDA(cols.ensure(sizeof(int32_t) * nhops));
        if (kind == HONEYCOMB)
            honeycomb_hops_kernel<<<grid_for(3 * nsub0), kThreads, 0, stream>>>(
                hp, nsub0, flat.as<int32_t>(), bits.as<int32_t>(), pos.as<int32_t>(), fin.as<int32_t>(),
                rows.as<int32_t>(), cols.as<int32_t>());
        else
            cubic_hops_kernel<<<grid_for(nhops), kThreads, 0, stream>>>(L, nsites, rows.as<int32_t>(),
                                                                        cols.as<int32_t>());
        ++launches;
        LAT_CUDA(cudaGetLastError());
        LAT_CUDA(cudaMemcpyAsync(hrows, rows.p, sizeof(int32_t) * nhops, cudaMemcpyDeviceToHost, stream));
        LAT_CUDA(cudaMemcpyAsync(hcols, cols.p, sizeof(int32_t) * nhops, cudaMemcpyDeviceToHost, stream));
        LAT_CUDA(cudaStreamSynchronize(stream));
        rows.release();
        cols.release();
        return KPM_OK;
    }

    template<class R, int NC>
    int csr(void const* hop_one, void const* hop_values, void const* onsite_h, int32_t* o_indptr, int32_t* o_indices,
            void* o_values, int64_t capacity, int64_t* nnz) {
        size_t const es = sizeof(R) * NC;
        Val<R, NC> hop_const{};
        if (hop_one) {
            for (int k = 0; k < NC; ++k) hop_const.c[k] = static_cast<R const*>(hop_one)[k];
        }
        LAT_CUDA(cudaEventRecord(ev0, stream));
        R const* d_hop = nullptr;
        if (hop_values && nhops > 0) {
            LAT_CUDA(hopv.ensure(es * nhops));
            LAT_CUDA(cudaMemcpyAsync(hopv.p, hop_values, es * nhops, cudaMemcpyHostToDevice, stream));
            d_hop = hopv.as<R>();
        }
        R const* d_onsite = nullptr;
        if (onsite_h && nsites > 0) {
            LAT_CUDA(onsite.ensure(es * nsites));
            LAT_CUDA(cudaMemcpyAsync(onsite.p, onsite_h, es * nsites, cudaMemcpyHostToDevice, stream));
            d_onsite = onsite.as<R>();
        }
        LAT_CUDA(counts.ensure(sizeof(int32_t) * (nsites + 1)));
        LAT_CUDA(indptr.ensure(sizeof(int32_t) * (nsites + 1)));
        LAT_CUDA(cudaMemsetAsync(counts.p, 0, sizeof(int32_t) * (nsites + 1), stream));
        if (nsites > 0) {
            if (kind == HONEYCOMB)
                honeycomb_counts_kernel<R, NC><<<grid_for(nsites), kThreads, 0, stream>>>(
                    hp, nsites, nsub0, flat.as<int32_t>(), valid.as<int32_t>(), bits.as<int32_t>(), d_onsite,
                    counts.as<int32_t>());
            else
                cubic_counts_kernel<R, NC><<<grid_for(nsites), kThreads, 0, stream>>>(nsites, d_onsite,
                                                                                      counts.as<int32_t>());
            ++launches;
            LAT_CUDA(cudaGetLastError());
        }
        int64_t total_nnz = 0;
        LAT_CHECK(scan(counts.as<int32_t>(), indptr.as<int32_t>(), nsites + 1, &total_nnz));
        if (total_nnz > capacity) return fail(KPM_ERR_VALUE, "kpm_lattice_csr: capacity is smaller than the entry count");
        LAT_CUDA(indices.ensure(sizeof(int32_t) * total_nnz));
        LAT_CUDA(values.ensure(es * total_nnz));
        if (nsites > 0) {
            if (kind == HONEYCOMB)
                honeycomb_fill_kernel<R, NC><<<grid_for(nsites), kThreads, 0, stream>>>(
                    hp, nsites, nsub0, flat.as<int32_t>(), valid.as<int32_t>(), fin.as<int32_t>(), bits.as<int32_t>(),
                    pos.as<int32_t>(), d_hop, hop_const, d_onsite, indptr.as<int32_t>(), indices.as<int32_t>(),
                    values.as<R>());
            else
                cubic_fill_kernel<R, NC><<<grid_for(nsites), kThreads, 0, stream>>>(
                    L, nsites, hop_const, d_onsite, indptr.as<int32_t>(), indices.as<int32_t>(), values.as<R>());
            ++launches;
            LAT_CUDA(cudaGetLastError());
        }
        LAT_CUDA(cudaEventRecord(ev1, stream));
        LAT_CUDA(cudaMemcpyAsync(o_indptr, indptr.p, sizeof(int32_t) * (nsites + 1), cudaMemcpyDeviceToHost, stream));
        if (total_nnz > 0) {
            LAT_CUDA(cudaMemcpyAsync(o_indices, indices.p, sizeof(int32_t) * total_nnz, cudaMemcpyDeviceToHost, stream));
            LAT_CUDA(cudaMemcpyAsync(o_values, values.p, es * total_nnz, cudaMemcpyDeviceToHost, stream));
        }
        LAT_CUDA(cudaStreamSynchronize(stream));
        csr_time = elapsed();
        *nnz = total_nnz;
        indices.release();
        values.release();
        hopv.release();
        onsite.release();
        return KPM_OK;
    }
};

// ====================================================================== C ABI
extern "C" int kpm_lattice_honeycomb(const kpm_honeycomb* params, const float* vertices, int32_t num_vertices,
                                     kpm_lattice** out) {
    if (!out) return fail(KPM_ERR_VALUE, "kpm_lattice_honeycomb: null output handle");
    *out = nullptr;
    if (!params || !vertices) return fail(KPM_ERR_VALUE, "kpm_lattice_honeycomb: null argument");
    if (params->s0 < 1 || params->s1 < 1) return fail(KPM_ERR_VALUE, "kpm_lattice_honeycomb: foundation size must be positive");
    if (2 * int64_t(params->s0) * params->s1 > INT32_MAX)
        return fail(KPM_ERR_VALUE, "kpm_lattice_honeycomb: the foundation exceeds int32 indices");
    if (num_vertices < 1 || num_vertices > (1 << 20))
        return fail(KPM_ERR_VALUE, "kpm_lattice_honeycomb: num_vertices must be in [1, 2^20]");
    if (params->min_neighbors < 0) return fail(KPM_ERR_VALUE, "kpm_lattice_honeycomb: min_neighbors must be >= 0");
    std::unique_ptr<kpm_lattice> h(new kpm_lattice);
    h->kind = kpm_lattice::HONEYCOMB;
    Honey& p = h->hp;
    p.s0 = params->s0;
    p.s1 = params->s1;
    p.block = int64_t(p.s0) * p.s1;
    for (int c = 0; c < 3; ++c) {
        p.origin[c] = params->origin[c];
        p.a1[c] = params->a1[c];
        p.a2[c] = params->a2[c];
        p.sub[0][c] = params->sub[0][c];
        p.sub[1][c] = params->sub[1][c];
    }
    for (int k = 0; k < 3; ++k) {
        p.hop[k][0] = params->hop[k][0];
        p.hop[k][1] = params->hop[k][1];
    }
    LAT_CHECK(h->init());
    LAT_CHECK(h->build_honeycomb(vertices, num_vertices, params->min_neighbors));
    *out = h.release();
    return KPM_OK;
}

extern "C" int kpm_lattice_cubic(int32_t L, kpm_lattice** out) {
    if (!out) return fail(KPM_ERR_VALUE, "kpm_lattice_cubic: null output handle");
    *out = nullptr;
    if (L < 3) return fail(KPM_ERR_VALUE, "kpm_lattice_cubic: L must be >= 3");
    if (7 * int64_t(L) * L * L > INT32_MAX) return fail(KPM_ERR_VALUE, "kpm_lattice_cubic: the lattice exceeds int32 indices");
    std::unique_ptr<kpm_lattice> h(new kpm_lattice);
    h->kind = kpm_lattice::CUBIC;
    h->L = L;
    LAT_CHECK(h->init());
    LAT_CHECK(h->build_cubic());
    *out = h.release();
    return KPM_OK;
}

extern "C" int kpm_lattice_sizes(const kpm_lattice* h, int64_t* num_sites, int64_t* num_sub0, int64_t* num_hoppings,
                                 int64_t* max_nnz) {
    if (!h) return fail(KPM_ERR_VALUE, "kpm_lattice_sizes: null handle");
    if (num_sites) *num_sites = h->nsites;
    if (num_sub0) *num_sub0 = h->nsub0;
    if (num_hoppings) *num_hoppings = h->nhops;
    if (max_nnz) *max_nnz = h->kind == kpm_lattice::HONEYCOMB ? 2 * h->nhops + h->nsites : 7 * h->nsites;
    return KPM_OK;
}

extern "C" int kpm_lattice_sites(kpm_lattice* h, float* x, float* y, float* z) {
    if (!h || !x || !y || !z) return fail(KPM_ERR_VALUE, "kpm_lattice_sites: null argument");
    if (h->nsites == 0) return KPM_OK;
    size_t const bytes = sizeof(float) * h->nsites;
    LAT_CUDA(cudaMemcpyAsync(x, h->x.p, bytes, cudaMemcpyDeviceToHost, h->stream));
    LAT_CUDA(cudaMemcpyAsync(y, h->y.p, bytes, cudaMemcpyDeviceToHost, h->stream));
    LAT_CUDA(cudaMemcpyAsync(z, h->z.p, bytes, cudaMemcpyDeviceToHost, h->stream));
    LAT_CUDA(cudaStreamSynchronize(h->stream));
    return KPM_OK;
}

extern "C" int kpm_lattice_hoppings(kpm_lattice* h, int32_t* rows, int32_t* cols) {
    if (!h || ((!rows || !cols) && h->nhops > 0)) return fail(KPM_ERR_VALUE, "kpm_lattice_hoppings: null argument");
    return h->hoppings(rows, cols);
}

extern "C" int kpm_lattice_csr(kpm_lattice* h, int32_t dtype, const void* hopping, const void* hopping_values,
                               const void* onsite, int32_t* indptr, int32_t* indices, void* values, int64_t capacity,
                               int64_t* nnz) {
    if (!h || !indptr || !nnz || ((!indices || !values) && capacity > 0))
        return fail(KPM_ERR_VALUE, "kpm_lattice_csr: null argument");
    if (!hopping && !hopping_values) return fail(KPM_ERR_VALUE, "kpm_lattice_csr: give a hopping value or the hopping values");
    if (hopping && hopping_values) return fail(KPM_ERR_VALUE, "kpm_lattice_csr: give either a hopping value or the hopping values");
    if (hopping_values && h->kind == kpm_lattice::CUBIC)
        return fail(KPM_ERR_VALUE, "kpm_lattice_csr: the cubic lattice takes a single hopping value");
    return with_dtype(dtype, [&](auto r, auto nc) {
        using R = decltype(r);
        return h->csr<R, decltype(nc)::value>(hopping, hopping_values, onsite, indptr, indices, values, capacity, nnz);
    });
}

extern "C" int kpm_lattice_times(const kpm_lattice* h, double* build_time, double* csr_time, int64_t* launches) {
    if (!h) return fail(KPM_ERR_VALUE, "kpm_lattice_times: null handle");
    if (build_time) *build_time = h->build_time;
    if (csr_time) *csr_time = h->csr_time;
    if (launches) *launches = h->launches;
    return KPM_OK;
}

extern "C" int kpm_lattice_destroy(kpm_lattice* h) {
    delete h;
    return KPM_OK;
}
