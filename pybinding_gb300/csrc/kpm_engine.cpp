// Host side of the GB300 KPM engine: the C ABI of include/kpm_gb300.h.
//
// Responsibilities (the reference's kpm::Core + OptimizedHamiltonian + Bounds +
// Starter + DefaultCompute, re-designed around one device and one stream):
//   * keep the Hamiltonian (one system or a ragged batch of block-diagonal
//     systems) and the per-system spectral bounds / scale factors;
//   * build the scaled, BFS-reordered matrix H~ = 2 (H - b) / a of every system
//     (the reference's create_reordered, OptimizedHamiltonian.cpp:75-152) and
//     upload it as padded row-major ELL in the recursion precision;
//   * draw the reference's random starters with std::mt19937 (Starter.cpp:48-84);
//   * drive the recursion kernels (one launch per Chebyshev step covering every
//     system and vector batch), collect moments, damp and reconstruct on the GPU;
//   * run Lanczos in FP64 on the GPU with the tridiagonal eigenproblem solved on
//     the host by Sturm-sequence bisection.
#include "kpm_gb300.h"
#include "kpm_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>
#include <random>
#include <stdexcept>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

using kpm::Tile;

namespace {

thread_local std::string g_last_error;

struct KpmError : std::runtime_error {
    int code;
    KpmError(int c, std::string const& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void fail(int code, std::string const& msg) { throw KpmError(code, msg); }

#define KPM_CUDA(expr)                                                                              \
    do {                                                                                            \
        cudaError_t e_ = (expr);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            fail(KPM_ERR_CUDA, std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " + #expr); \
    } while (0)

template<class F>
int guarded(F&& f) {
    try {
        f();
        return KPM_OK;
    } catch (KpmError const& e) {
        g_last_error = e.what();
        return e.code;
    } catch (std::invalid_argument const& e) {
        g_last_error = e.what();
        return KPM_ERR_VALUE;
    } catch (std::bad_alloc const&) {
        g_last_error = "out of host memory";
        return KPM_ERR_RUNTIME;
    } catch (std::exception const& e) {
        g_last_error = e.what();
        return KPM_ERR_RUNTIME;
    }
}

// ------------------------------------------------------------------ device memory
struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DBuf() = default;
    DBuf(DBuf const&) = delete;
    DBuf& operator=(DBuf const&) = delete;
    ~DBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    void ensure(size_t n) {
        if (n <= bytes && p) return;
        release();
        if (n == 0) n = 16;
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            fail(KPM_ERR_CUDA, "device allocation of " + std::to_string(n) + " bytes failed: " + cudaGetErrorString(e));
        }
        bytes = n;
    }
    template<class T> T* as() const { return static_cast<T*>(p); }
};

// ------------------------------------------------------------------ scalar helpers
using cf = std::complex<float>;
using cd = std::complex<double>;

int scalar_bytes(int st) { return st == KPM_F32 ? 4 : (st == KPM_C128 ? 16 : 8); }
bool scalar_complex(int st) { return st == KPM_C64 || st == KPM_C128; }

template<class T> struct RealOf { using type = T; };
template<class T> struct RealOf<std::complex<T>> { using type = T; };
template<class T> using real_of = typename RealOf<T>::type;
template<class T> constexpr bool is_cplx_v = !std::is_same<T, real_of<T>>::value;

template<class T> cd to_cd(T v) { return cd(static_cast<double>(v), 0.0); }
template<> cd to_cd<cf>(cf v) { return cd(v.real(), v.imag()); }
template<> cd to_cd<cd>(cd v) { return v; }

template<class T> T from_cd(cd v);
template<> float from_cd<float>(cd v) { return static_cast<float>(v.real()); }
template<> double from_cd<double>(cd v) { return v.real(); }
template<> cf from_cd<cf>(cd v) { return cf(static_cast<float>(v.real()), static_cast<float>(v.imag())); }
template<> cd from_cd<cd>(cd v) { return v; }

// convert value of scalar type Tin to compute type Tc (real->complex allowed)
template<class Tc, class Tin> Tc convert(Tin v) {
    if constexpr (is_cplx_v<Tc>) {
        if constexpr (is_cplx_v<Tin>)
            return Tc(static_cast<real_of<Tc>>(v.real()), static_cast<real_of<Tc>>(v.imag()));
        else
            return Tc(static_cast<real_of<Tc>>(v), real_of<Tc>(0));
    } else {
        if constexpr (is_cplx_v<Tin>) return static_cast<Tc>(v.real());
        else return static_cast<Tc>(v);
    }
}

template<class F>
void with_scalar(int st, F&& f) {
    switch (st) {
        case KPM_F32: f(float{}); break;
        case KPM_F64: f(double{}); break;
        case KPM_C64: f(cf{}); break;
        case KPM_C128: f(cd{}); break;
        default: fail(KPM_ERR_VALUE, "unknown scalar type");
    }
}
template<class F>
void with_vtype(int vt, F&& f) {
    switch (vt) {
        case kpm::V_F32: f(float{}); break;
        case kpm::V_F64: f(double{}); break;
        case kpm::V_C64: f(cf{}); break;
        default: f(cd{}); break;
    }
}

// ------------------------------------------------------------------ scale and kernels
// kpm::Scale<double>(min, max) (kpm/Bounds.hpp:15-30): float constants as in the reference
struct ScaleAB { double a = 0, b = 0; };
ScaleAB make_scale(double emin, double emax) {
    constexpr float tol = 0.01f;
    ScaleAB s;
    s.a = 0.5f * (emax - emin) * (1 + tol);
    s.b = 0.5f * (emax + emin);
    if (std::abs(s.b / s.a) < 0.01f * tol) s.b = 0;
    return s;
}

constexpr float PI_F = 3.14159265358979323846f;  // the reference's pi constant is a float

int64_t round_moments(int64_t n) {
    if (n < 2) return 2;
    return n + ((4 - (n - 2) % 4) % 4);
}

std::vector<double> damping(int kernel, double lambda, int64_t M) {
    std::vector<double> g(static_cast<size_t>(M));
    double const N = static_cast<double>(M);
    double const pi = static_cast<double>(PI_F);
    for (int64_t i = 0; i < M; ++i) {
        double const n = static_cast<double>(i);
        if (kernel == KPM_KERNEL_JACKSON) {
            double const Np = N + 1;
            g[i] = ((Np - n) * std::cos(pi * n / Np) + std::sin(pi * n / Np) / std::tan(pi / Np)) / Np;
        } else if (kernel == KPM_KERNEL_LORENTZ) {
            g[i] = std::sinh(lambda * (1 - n / N)) / std::sinh(lambda);
        } else {
            g[i] = 1.0;
        }
    }
    return g;
}

int64_t required_moments(int kernel, double lambda, double scaled_broadening) {
    double const num = kernel == KPM_KERNEL_LORENTZ ? lambda : static_cast<double>(PI_F);
    return round_moments(static_cast<int64_t>(num / scaled_broadening) + 1);
}

// ------------------------------------------------------------------ tridiagonal extremes
// Extreme eigenvalues of the symmetric tridiagonal (alpha, beta[0..k-2]) by
// Sturm-sequence bisection: count(x) = #eigenvalues < x.
// Two counts in one pass: the two recurrences are independent, so interleaving them
// overlaps their dependent divisions; each count is computed exactly as alone.
void sturm_count2(std::vector<double> const& a, std::vector<double> const& b, double x0, double x1, int& c0, int& c1) {
    double const eps = std::numeric_limits<double>::epsilon();
    int n0 = 0, n1 = 0;
    double q0 = a[0] - x0, q1 = a[0] - x1;
    n0 += q0 < 0;
    n1 += q1 < 0;
    for (size_t i = 1; i < a.size(); ++i) {
        double const bb = b[i - 1] * b[i - 1];
        double const tiny = eps * (std::abs(b[i - 1]) + 1e-300);
        if (q0 == 0) q0 = tiny;
        if (q1 == 0) q1 = tiny;
        q0 = a[i] - x0 - bb / q0;
        q1 = a[i] - x1 - bb / q1;
        n0 += q0 < 0;
        n1 += q1 < 0;
    }
    c0 = n0;
    c1 = n1;
}

void tridiagonal_extremes(std::vector<double> const& a, std::vector<double> const& b, double& mn, double& mx) {
    size_t const k = a.size();
    double lo = std::numeric_limits<double>::max(), hi = std::numeric_limits<double>::lowest();
    for (size_t i = 0; i < k; ++i) {
        double r = 0;
        if (i > 0) r += std::abs(b[i - 1]);
        if (i + 1 < k) r += std::abs(b[i]);
        lo = std::min(lo, a[i] - r);
        hi = std::max(hi, a[i] + r);
    }
    double const span = std::max(hi - lo, 1e-300);
    lo -= 1e-12 * span;
    hi += 1e-12 * span;
    // Bisection for the smallest x with count(x) > target, for target 0 (minimum) and
    // k - 1 (maximum), both brackets advanced in the same pass; each stops on its own.
    int const target[2] = {0, static_cast<int>(k) - 1};
    double l[2] = {lo, lo}, h[2] = {hi, hi};
    int it[2] = {0, 0};
    auto open = [&](int j) {
        return it[j] < 200 && h[j] - l[j] > 1e-15 * std::max(std::abs(l[j]), std::abs(h[j])) + 1e-300;
    };
    while (open(0) || open(1)) {
        bool const o0 = open(0), o1 = open(1);
        double const m0 = 0.5 * (l[0] + h[0]), m1 = 0.5 * (l[1] + h[1]);
        int c0, c1;
        sturm_count2(a, b, m0, m1, c0, c1);
        if (o0) { (c0 > target[0] ? h[0] : l[0]) = m0; ++it[0]; }
        if (o1) { (c1 > target[1] ? h[1] : l[1]) = m1; ++it[1]; }
    }
    mn = 0.5 * (l[0] + h[0]);
    mx = 0.5 * (l[1] + h[1]);
}

std::string with_suffix(double v) {
    char buf[64];
    char const* suf[] = {"", "K", "M", "G", "T", "P"};
    int i = 0;
    while (std::abs(v) >= 1000.0 && i < 5) { v /= 1000.0; ++i; }
    std::snprintf(buf, sizeof buf, i == 0 ? "%.0f%s" : "%.3g%s", v, suf[i]);
    return buf;
}

std::string pretty_time(double s) {
    char buf[64];
    if (s < 1e-3) std::snprintf(buf, sizeof buf, "%.1f us", s * 1e6);
    else if (s < 1) std::snprintf(buf, sizeof buf, "%.2f ms", s * 1e3);
    else std::snprintf(buf, sizeof buf, "%.3f s", s);
    return buf;
}

// Host threads for the setup work of the engine call running on this thread: the engine's
// num_threads (kpm::DefaultCompute's num_threads, cppmodule/src/kpm.cpp:14), 0 = all cores.
thread_local int tl_host_threads = 0;
struct HostThreads {
    int saved;
    explicit HostThreads(int n) : saved(tl_host_threads) { tl_host_threads = n; }
    ~HostThreads() { tl_host_threads = saved; }
};

// Runs f(0 .. count-1) on up to hardware_concurrency (or num_threads) threads (host-side setup work).
template<class F>
void parallel_for(int64_t count, F&& f) {
    int64_t hw = std::thread::hardware_concurrency();
    if (tl_host_threads > 0) hw = std::min<int64_t>(hw, tl_host_threads);
    int64_t const nt = std::max<int64_t>(1, std::min<int64_t>(count, hw));
    if (nt <= 1) {
        for (int64_t i = 0; i < count; ++i) f(i);
        return;
    }
    std::atomic<int64_t> next{0};
    std::vector<std::thread> pool;
    for (int64_t t = 0; t < nt; ++t)
        pool.emplace_back([&] {
            for (int64_t i = next++; i < count; i = next++) f(i);
        });
    for (auto& th : pool) th.join();
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

// ====================================================================== engine
struct kpm_engine {
    // input
    int stype = KPM_F32;
    kpm_config cfg{};
    int vtype = kpm::V_F32;
    int64_t rows = 0;
    int nsys = 1;
    std::vector<int64_t> sys_off;           // nsys + 1
    std::vector<int32_t> indptr, indices;   // global CSR, global column indices
    std::vector<unsigned char> values;      // stype

    // per system bounds
    struct Sys {
        bool have_bounds = false;
        double emin = 0, emax = 0;
        int loops = 0;
    };
    std::vector<Sys> sys;

    // current optimization (reordered, scaled device matrix)
    bool opt_valid = false;
    std::vector<int32_t> opt_src, opt_dest;  // target indices (system 0) or {0} for all systems
    std::vector<int32_t> map;                // original global row -> reordered global row
    std::vector<int32_t> slices;             // SliceMap borders (system 0)
    int64_t src_offset = 0, dest_offset = 0;
    std::vector<int32_t> idx_src, idx_dest;  // reordered target indices
    int W = 0;
    int64_t opt_nnz = 0;                     // reordered CSR non-zeros (all systems)
    DBuf d_col, d_val, d_map, d_sysoff;
    DBuf d_val_real;          // real-valued copy of a complex H~ whose values are all real
    bool real_values = false;

    // Lanczos device state
    bool lz_uploaded = false;
    DBuf d_lip, d_lix, d_lval, d_lv0, d_lv1, d_ltiles, d_lab, d_lpart, d_lsys;
    int lz_tiles = 0;

    // recursion buffers
    DBuf d_x0, d_x1, d_acc, d_tiles, d_mu, d_mu_avg, d_stage, d_pos, d_gamma, d_energy, d_out;
    std::vector<int32_t> h_col;  // host copy of the device ELL column indices

    // two-steps-per-launch state: one partition per candidate tile height
    struct PairPlan {
        int rows_per_tile = 0;
        int num_tiles = 0;
        DBuf d_tiles, d_items, d_band, d_flags;
    };
    std::vector<std::unique_ptr<PairPlan>> pair_plans;
    int pair_key_nbatch = -1, pair_key_lpr = -1;
    int64_t pair_key_rows = -1;
    int pair_seq = 0;
    DBuf d_pair_counters, d_pair_error;

    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    // stats of the last calculation
    kpm_stats st{};
    double calc_time = 0;
    bool last_bounds_lanczos = false;

    // The single-step recursion of the last diagonal call as a CUDA graph (one node per
    // step), replayed while every pointer and size it captured is unchanged.
    struct RecursionGraphKey {
        void const *x0, *x1, *acc, *tiles, *col, *val;
        int64_t half, bstride, step_acc;
        int ntiles, vtype, E, LPR, nbatch, unroll, W, prefetch;
        int32_t row_limit;
        bool real_matrix;
        bool operator==(RecursionGraphKey const& o) const { return std::memcmp(this, &o, sizeof o) == 0; }
    };
    RecursionGraphKey graph_key{};
    cudaGraphExec_t graph_exec = nullptr;
    // The GPU can dereference pageable host memory through the host's page tables (address
    // translation services on Grace): kernels then read caller-provided host buffers in place.
    int host_direct = -1;
    bool host_reads_direct() {
        if (host_direct < 0) {
            int dev = 0, pageable = 0, host_tables = 0;
            KPM_CUDA(cudaGetDevice(&dev));
            KPM_CUDA(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev));
            KPM_CUDA(cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev));
            host_direct = (pageable && host_tables) ? 1 : 0;
        }
        return host_direct == 1;
    }

    // A device-readable view of a host buffer for a kernel on `stream`: the buffer itself where
    // the GPU reads host memory in place, else a copy in d_stage. The host buffer must stay
    // unchanged until the stream has consumed it.
    void const* device_view(void const* host, size_t bytes) {
        if (host_reads_direct()) return host;
        d_stage.ensure(bytes);
        KPM_CUDA(cudaMemcpyAsync(d_stage.p, host, bytes, cudaMemcpyHostToDevice, stream));
        return d_stage.p;
    }

    // Host-to-device copy of a host buffer on `stream`: where the GPU reads host memory through
    // the host page tables, a copy kernel reads it in place (a pageable cudaMemcpyAsync is staged
    // through bounce buffers at a fraction of the link's rate); elsewhere cudaMemcpyAsync. The
    // host buffer must stay unchanged until the stream has run the copy.
    void upload_host(void* dst, void const* src, size_t bytes) {
        if (bytes == 0) return;
        bool const aligned = ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) % 16) == 0;
        if (host_reads_direct() && aligned) KPM_CUDA(kpm::launch_copy(dst, src, bytes, stream));
        else KPM_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream));
    }

    std::vector<unsigned char> h_starters, h_starters_right;  // host starters the engine generates

    // Progress of the stochastic DOS (DefaultCompute::progress_start/update/finish,
    // kpm/default/Compute.cpp:64-87,133-144): fn(-1, total) before the recursion, increments
    // adding up to `total` vectors as segments of the recursion complete, fn(total, total) at the
    // end; called on the calling thread, which waits on the segments' events.
    kpm_progress_fn progress_fn = nullptr;
    void* progress_user = nullptr;
    int64_t progress_total = 0;  // > 0 while a DOS call reports progress
    static constexpr int kProgressSegments = 8;
    cudaEvent_t progress_ev[kProgressSegments] = {};
    void progress(int64_t delta) {
        if (progress_fn && progress_total > 0) progress_fn(delta, progress_total, progress_user);
    }

    void drop_graph() {
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        graph_exec = nullptr;
    }

    ~kpm_engine() {
        drop_graph();
        for (auto& ev : progress_ev)
            if (ev) cudaEventDestroy(ev);
        if (ev_t0) cudaEventDestroy(ev_t0);
        if (ev_t1) cudaEventDestroy(ev_t1);
        if (ev_u0) cudaEventDestroy(ev_u0);
        if (ev_u1) cudaEventDestroy(ev_u1);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }

    int64_t sys_rows(int s) const { return sys_off[s + 1] - sys_off[s]; }

    // The device is touched on first use, so that argument checks and host-only
    // entry points work (and fail cleanly) without a GPU.
    void ensure_device() {
        if (stream) return;
        int dev_count = 0;
        cudaError_t e = cudaGetDeviceCount(&dev_count);
        if (e != cudaSuccess || dev_count < 1) {
            cudaGetLastError();
            fail(KPM_ERR_CUDA, std::string("no CUDA device available: ") + cudaGetErrorString(e));
        }
        KPM_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        KPM_CUDA(cudaEventCreate(&ev0));
        KPM_CUDA(cudaEventCreate(&ev1));
        KPM_CUDA(cudaEventCreate(&ev_t0));
        KPM_CUDA(cudaEventCreate(&ev_t1));
        KPM_CUDA(cudaEventCreate(&ev_u0));
        KPM_CUDA(cudaEventCreate(&ev_u1));
    }

    void set_h(int st_, int64_t n, int32_t const* ip, int32_t const* ix, void const* v, int ns, int64_t const* offs) {
        if (n <= 0) fail(KPM_ERR_VALUE, "the Hamiltonian must have at least one row");
        if (!ip || !ix || !v) fail(KPM_ERR_VALUE, "null Hamiltonian arrays");
        if (st_ < KPM_F32 || st_ > KPM_C128) fail(KPM_ERR_VALUE, "unknown scalar type");
        if (ns < 1) fail(KPM_ERR_VALUE, "num_systems must be >= 1");
        if (n > std::numeric_limits<int32_t>::max()) fail(KPM_ERR_VALUE, "too many rows for int32 indices");
        std::vector<int64_t> off(ns + 1);
        if (ns == 1 || !offs) {
            if (ns != 1) fail(KPM_ERR_VALUE, "system_offsets required for num_systems > 1");
            off = {0, n};
        } else {
            off.assign(offs, offs + ns + 1);
            if (off[0] != 0 || off[ns] != n) fail(KPM_ERR_VALUE, "system_offsets must start at 0 and end at rows");
            for (int s = 0; s < ns; ++s)
                if (off[s + 1] <= off[s]) fail(KPM_ERR_VALUE, "system_offsets must be strictly increasing");
        }
        int64_t const nnz = ip[n];
        if (ip[0] != 0 || nnz < 0) fail(KPM_ERR_VALUE, "invalid CSR indptr");
        for (int64_t r = 0; r < n; ++r)
            if (ip[r + 1] < ip[r]) fail(KPM_ERR_VALUE, "invalid CSR indptr (decreasing)");
        // columns in range, sorted, within the row's own system (block diagonal)
        int s = 0;
        for (int64_t r = 0; r < n; ++r) {
            while (r >= off[s + 1]) ++s;
            for (int64_t k = ip[r]; k < ip[r + 1]; ++k) {
                int64_t const c = ix[k];
                if (c < off[s] || c >= off[s + 1])
                    fail(KPM_ERR_VALUE, "CSR column index out of range (or outside its system block)");
                if (k > ip[r] && ix[k - 1] >= c) fail(KPM_ERR_VALUE, "CSR column indices must be sorted and unique");
            }
        }
        // Hamiltonian.hpp:133-140
        size_t const sb = static_cast<size_t>(scalar_bytes(st_));
        bool finite = true;
        with_scalar(st_, [&](auto z) {
            using T = decltype(z);
            auto const* p = static_cast<T const*>(v);
            for (int64_t k = 0; k < nnz && finite; ++k) {
                cd const c = to_cd(p[k]);
                if (!std::isfinite(c.real()) || !std::isfinite(c.imag())) finite = false;
            }
        });
        if (!finite)
            fail(KPM_ERR_RUNTIME, "The Hamiltonian contains invalid values: NaN or INF.\n"
                                  "Check the lattice and/or modifier functions.");
        stype = st_;
        rows = n;
        nsys = ns;
        sys_off = off;
        indptr.assign(ip, ip + n + 1);
        indices.assign(ix, ix + nnz);
        values.assign(static_cast<unsigned char const*>(v), static_cast<unsigned char const*>(v) + nnz * sb);
        sys.assign(ns, Sys{});
        if (cfg.min_energy != cfg.max_energy)
            for (auto& x : sys) { x.have_bounds = true; x.emin = cfg.min_energy; x.emax = cfg.max_energy; }
        opt_valid = false;
        lz_uploaded = false;
        // recursion precision (KPM_PREC_*)
        bool const dbl = cfg.precision == KPM_PREC_FP64 ||
                         (cfg.precision == KPM_PREC_AUTO && (st_ == KPM_F64 || st_ == KPM_C128));
        bool const cpx = scalar_complex(st_);
        vtype = cpx ? (dbl ? kpm::V_C128 : kpm::V_C64) : (dbl ? kpm::V_F64 : kpm::V_F32);
    }

    // ---------------------------------------------------------------- Lanczos (FP64, GPU)
    void upload_lanczos() {
        if (lz_uploaded) return;
        ensure_device();
        bool const cpx = scalar_complex(stype);
        size_t const es = cpx ? 16 : 8;
        int64_t const nnz = indptr[rows];
        std::vector<unsigned char> vals(static_cast<size_t>(nnz) * es);
        with_scalar(stype, [&](auto z) {
            using T = decltype(z);
            auto const* p = reinterpret_cast<T const*>(values.data());
            int64_t const chunk = 1 << 20;
            parallel_for((nnz + chunk - 1) / chunk, [&](int64_t c) {
                int64_t const k1 = std::min(nnz, (c + 1) * chunk);
                if (cpx) {
                    auto* o = reinterpret_cast<cd*>(vals.data());
                    for (int64_t k = c * chunk; k < k1; ++k) o[k] = to_cd(p[k]);
                } else {
                    auto* o = reinterpret_cast<double*>(vals.data());
                    for (int64_t k = c * chunk; k < k1; ++k) o[k] = to_cd(p[k]).real();
                }
            });
        });
        d_lip.ensure(sizeof(int32_t) * (rows + 1));
        d_lix.ensure(sizeof(int32_t) * std::max<int64_t>(nnz, 1));
        d_lval.ensure(std::max<size_t>(vals.size(), 16));
        upload_host(d_lip.p, indptr.data(), sizeof(int32_t) * (rows + 1));
        if (nnz > 0) {
            upload_host(d_lix.p, indices.data(), sizeof(int32_t) * nnz);
            upload_host(d_lval.p, vals.data(), vals.size());
        }
        std::vector<Tile> tiles;
        std::vector<int32_t> sys_tiles{0};  // tiles of system s: sys_tiles[s] .. sys_tiles[s + 1] - 1
        for (int s = 0; s < nsys; ++s) {
            for (int64_t r = sys_off[s]; r < sys_off[s + 1]; r += 2048)
                tiles.push_back({static_cast<int32_t>(r), static_cast<int32_t>(std::min(sys_off[s + 1], r + 2048)), s, 0});
            sys_tiles.push_back(static_cast<int32_t>(tiles.size()));
        }
        lz_tiles = static_cast<int>(tiles.size());
        d_ltiles.ensure(sizeof(Tile) * tiles.size());
        KPM_CUDA(cudaMemcpyAsync(d_ltiles.p, tiles.data(), sizeof(Tile) * tiles.size(), cudaMemcpyHostToDevice, stream));
        d_lpart.ensure(sizeof(double) * tiles.size());
        d_lsys.ensure(sizeof(int32_t) * sys_tiles.size());
        KPM_CUDA(cudaMemcpyAsync(d_lsys.p, sys_tiles.data(), sizeof(int32_t) * sys_tiles.size(), cudaMemcpyHostToDevice,
                                 stream));
        d_lv0.ensure(es * rows);
        d_lv1.ensure(es * rows);
        d_lab.ensure(sizeof(double) * 3 * nsys);
        KPM_CUDA(cudaStreamSynchronize(stream));
        lz_uploaded = true;
    }

    // Bounds for every system that lacks them: compute/lanczos.hpp:101-154 in FP64.
    void compute_bounds() {
        std::vector<int> todo;
        for (int s = 0; s < nsys; ++s)
            if (!sys[s].have_bounds) todo.push_back(s);
        if (todo.empty()) return;
        double const t0 = now_s();
        upload_lanczos();
        bool const cpx = scalar_complex(stype);
        size_t const es = cpx ? 16 : 8;
        // start vectors: U[0,1) from a fresh default mt19937 per system in H's real type, normalized
        std::vector<unsigned char> v1(es * rows);
        parallel_for(nsys, [&](int64_t s) {  // one generator per system: independent
            std::mt19937 gen;
            int64_t const n = sys_rows(s);
            std::vector<double> u(static_cast<size_t>(n));
            if (stype == KPM_F32 || stype == KPM_C64) {
                std::uniform_real_distribution<float> dist;
                for (auto& x : u) x = dist(gen);
            } else {
                std::uniform_real_distribution<double> dist;
                for (auto& x : u) x = dist(gen);
            }
            double nrm = 0;
            for (auto x : u) nrm += x * x;
            nrm = std::sqrt(nrm);
            for (int64_t i = 0; i < n; ++i) {
                double const val = nrm > 0 ? u[i] / nrm : 0.0;
                if (cpx) reinterpret_cast<cd*>(v1.data())[sys_off[s] + i] = cd(val, 0);
                else reinterpret_cast<double*>(v1.data())[sys_off[s] + i] = val;
            }
        });
        upload_host(d_lv1.p, v1.data(), v1.size());
        KPM_CUDA(cudaMemsetAsync(d_lv0.p, 0, es * rows, stream));
        std::vector<std::vector<double>> alpha(nsys), beta(nsys);
        std::vector<double> prev_min(nsys, std::numeric_limits<double>::max());
        std::vector<double> prev_max(nsys, std::numeric_limits<double>::lowest());
        std::vector<char> done(nsys, 1);
        for (int s : todo) done[s] = 0;
        double const precision = static_cast<double>(static_cast<float>(cfg.lanczos_precision)) / 100;
        // kLzBlock iterations run on the device between host checks: the beta of an iteration
        // is computed on the device from the previous squared norm, and the host then replays
        // the convergence test iteration by iteration on the downloaded (alpha, |v|^2), so the
        // result and the loop count are those of checking after every iteration; systems that
        // converged early in a block just run a few iterations nobody reads
        constexpr int kLzBlock = 16;
        size_t const slot = static_cast<size_t>(nsys);
        d_lab.ensure(sizeof(double) * slot * (1 + 2 * kLzBlock));
        double* const dprev = d_lab.as<double>();           // |v|^2 of the iteration before the block
        double* const dblock = dprev + slot;                 // per iteration j: alpha_j, |v|^2_j
        KPM_CUDA(cudaMemsetAsync(dprev, 0, sizeof(double) * slot, stream));
        std::vector<double> hb(2 * kLzBlock * slot);
        void* v0 = d_lv0.p;
        void* v1d = d_lv1.p;
        std::vector<int> open;
        for (int it0 = 0; it0 < 1000; it0 += kLzBlock) {
            int const nb = std::min(kLzBlock, 1000 - it0);
            KPM_CUDA(cudaMemsetAsync(dblock, 0, sizeof(double) * 2 * slot * nb, stream));
            for (int j = 0; j < nb; ++j) {
                double const* np = j == 0 ? dprev : dblock + (2 * j - 1) * slot;
                double* al = dblock + 2 * j * slot;
                double* nr = al + slot;
                KPM_CUDA(kpm::launch_lanczos_a(cpx, d_lip.as<int32_t>(), d_lix.as<int32_t>(), d_lval.p, v1d, v0,
                                               d_ltiles.as<Tile>(), lz_tiles, np, d_lpart.as<double>(),
                                               d_lsys.as<int32_t>(), nsys, al, stream));
                KPM_CUDA(kpm::launch_lanczos_b(cpx, v1d, v0, d_ltiles.as<Tile>(), lz_tiles, al, d_lpart.as<double>(),
                                               d_lsys.as<int32_t>(), nsys, nr, stream));
                KPM_CUDA(kpm::launch_lanczos_c(cpx, v0, d_ltiles.as<Tile>(), lz_tiles, nr, stream));
                std::swap(v0, v1d);
            }
            KPM_CUDA(cudaMemcpyAsync(hb.data(), dblock, sizeof(double) * 2 * slot * nb, cudaMemcpyDeviceToHost, stream));
            KPM_CUDA(cudaMemcpyAsync(dprev, dblock + (2 * nb - 1) * slot, sizeof(double) * slot,
                                     cudaMemcpyDeviceToDevice, stream));
            KPM_CUDA(cudaStreamSynchronize(stream));
            open.clear();
            for (int s = 0; s < nsys; ++s)
                if (!done[s]) open.push_back(s);
            // systems are independent: each replays its iterations of the block on its own
            auto replay = [&](int64_t q) {
                int const s = open[q];
                for (int j = 0; j < nb && !done[s]; ++j) {
                    alpha[s].push_back(hb[2 * j * slot + s]);
                    beta[s].push_back(std::sqrt(hb[(2 * j + 1) * slot + s]));
                    double mn, mx;
                    tridiagonal_extremes(alpha[s], beta[s], mn, mx);
                    bool const cmin = std::abs((prev_min[s] - mn) / mn) < precision;
                    bool const cmax = std::abs((prev_max[s] - mx) / mx) < precision;
                    if (cmin && cmax) {
                        done[s] = 1;
                        sys[s].have_bounds = true;
                        sys[s].emin = mn;
                        sys[s].emax = mx;
                        sys[s].loops = it0 + j;
                    }
                    prev_min[s] = mn;
                    prev_max[s] = mx;
                }
            };
            if (open.size() > 1) parallel_for(static_cast<int64_t>(open.size()), replay);
            else if (!open.empty()) replay(0);
            bool all = true;
            for (int s = 0; s < nsys; ++s) all = all && done[s];
            if (all) {
                st.bounds_time = now_s() - t0;
                st.lanczos_loops = sys[todo.front()].loops;
                last_bounds_lanczos = true;
                return;
            }
        }
        fail(KPM_ERR_RUNTIME, "Lanczos algorithm did not converge for the min/max eigenvalues.");
    }

    ScaleAB scale(int s) {
        compute_bounds();
        return make_scale(sys[s].emin, sys[s].emax);
    }

    // ---------------------------------------------------------------- optimization
    // BFS reorder + scale of one system into the compute type Tc, appended to the
    // global reordered CSR (OptimizedHamiltonian.cpp:75-152 / 55-72 semantics).
    template<class Tc, class Tin>
    void reorder_system(int s, std::vector<int32_t> const& src_local, ScaleAB sc, bool reorder,
                        std::vector<int32_t>& oip, std::vector<int32_t>& oix, std::vector<Tc>& oval,
                        std::vector<int32_t>* borders_out) {
        using R = real_of<Tc>;
        int64_t const off = sys_off[s], n = sys_rows(s);
        auto const* hv = reinterpret_cast<Tin const*>(values.data());
        R const a = static_cast<R>(sc.a), b = static_cast<R>(sc.b);
        R const inv_a = R{2 / a};
        std::vector<int32_t> order;
        order.reserve(n);
        std::vector<int32_t> local(n, -1);
        std::vector<int32_t> borders{1};
        if (reorder) {
            order.push_back(src_local[0]);
            local[src_local[0]] = 0;
        } else {
            for (int64_t i = 0; i < n; ++i) { order.push_back(static_cast<int32_t>(i)); local[i] = static_cast<int32_t>(i); }
        }
        std::vector<std::pair<int32_t, Tc>> row_buf;
        int32_t next_unvisited = 0;
        for (int64_t nr = 0; nr < n; ++nr) {
            if (nr == static_cast<int64_t>(order.size())) {
                // the breadth-first search has exhausted the target's connected component (the
                // reference assumes a connected graph and would read past its queue here): continue
                // from the first row not reached yet, as a new component
                while (local[next_unvisited] >= 0) ++next_unvisited;
                local[next_unvisited] = static_cast<int32_t>(order.size());
                order.push_back(next_unvisited);
            }
            int32_t const orow = order[nr];
            row_buf.clear();
            bool diag = false;
            for (int32_t k = indptr[off + orow]; k < indptr[off + orow + 1]; ++k) {
                int32_t const ocol = static_cast<int32_t>(indices[k] - off);
                if (local[ocol] < 0) {
                    local[ocol] = static_cast<int32_t>(order.size());
                    order.push_back(ocol);
                }
                Tc v;
                if (reorder) {  // value * (2/a) - b * (2/a) on the diagonal
                    v = convert<Tc>(hv[k]) * inv_a;
                    if (ocol == orow) { v -= b * inv_a; diag = true; }
                } else {        // (value - b) * (2/a)
                    v = convert<Tc>(hv[k]);
                    if (ocol == orow) { if (b != R(0)) v -= b; diag = true; }
                    v = v * (R{2} / a);
                }
                row_buf.push_back({local[ocol], v});
            }
            if (b != R(0) && !diag) {
                Tc v = reorder ? Tc(-b * inv_a) : (Tc(R(0)) - Tc(b)) * (R{2} / a);
                row_buf.push_back({static_cast<int32_t>(nr), v});
            }
            std::sort(row_buf.begin(), row_buf.end(),
                      [](std::pair<int32_t, Tc> const& x, std::pair<int32_t, Tc> const& y) { return x.first < y.first; });
            for (auto const& p : row_buf) {
                oix.push_back(static_cast<int32_t>(p.first + off));
                oval.push_back(p.second);
            }
            oip.push_back(static_cast<int32_t>(oix.size()));
            if (reorder && nr == borders.back() - 1) borders.push_back(static_cast<int32_t>(order.size()));
        }
        for (int64_t i = 0; i < n; ++i) map[off + i] = static_cast<int32_t>(local[i] + off);
        if (borders_out) {
            if (reorder) {
                borders.pop_back();
                *borders_out = borders;
            } else {
                *borders_out = {static_cast<int32_t>(n)};
            }
        }
    }

    bool reorders() const { return cfg.optimal_size || cfg.interleaved; }

    // Optimize every system for source row 0 (DOS, moments, conductivity) or system 0
    // for (src, dest) targets; upload the padded ELL in the recursion type.
    void optimize(std::vector<int32_t> const& src, std::vector<int32_t> const& dest) {
        if (opt_valid && src == opt_src && dest == opt_dest) return;
        ensure_device();
        double const t0 = now_s();
        compute_bounds();
        map.assign(rows, 0);
        W = 0;
        // H~ in FP64 (the scaled values of create_reordered evaluated in double), then stored in the
        // recursion type: FP64 as is, FP32 as (hi, lo) pairs
        bool const cpx = kpm::vtype_complex(vtype);
        // systems are independent: reorder them in parallel into their own buffers, then write
        // each one's rows of the padded ELL, again in parallel
        std::vector<ScaleAB> scs(nsys);  // bounds (Lanczos on the GPU) before the threads start
        for (int s = 0; s < nsys; ++s) scs[s] = scale(s);
        std::vector<std::vector<int32_t>> sip(nsys), six(nsys);  // per system: row ends, global columns
        std::vector<std::vector<cd>> svc(cpx ? nsys : 0);
        std::vector<std::vector<double>> svr(cpx ? 0 : nsys);
        std::vector<int32_t> sys_w(nsys, 1);
        with_scalar(stype, [&](auto zi) {
            using Tin = decltype(zi);
            parallel_for(nsys, [&](int64_t s) {
                std::vector<int32_t> sl = (s == 0) ? src : std::vector<int32_t>{0};
                if (cpx)
                    reorder_system<cd, Tin>(static_cast<int>(s), sl, scs[s], reorders(), sip[s], six[s], svc[s],
                                            s == 0 ? &slices : nullptr);
                else
                    reorder_system<double, Tin>(static_cast<int>(s), sl, scs[s], reorders(), sip[s], six[s], svr[s],
                                                s == 0 ? &slices : nullptr);
                int32_t prev = 0;
                for (int32_t e : sip[s]) {
                    sys_w[s] = std::max(sys_w[s], e - prev);
                    prev = e;
                }
            });
        });
        for (int s = 0; s < nsys; ++s) W = std::max(W, sys_w[s]);
        int64_t total_nnz = 0;
        for (int s = 0; s < nsys; ++s) total_nnz += sip[s].empty() ? 0 : sip[s].back();
        int const vs = kpm::vtype_vs(vtype);
        std::vector<int32_t> col(static_cast<size_t>(rows) * W);
        // visit the entries of system s, row by row: f(row, slot, column, value) for stored
        // entries and pad(row, slot) for the padding slots up to W
        auto for_rows = [&](int64_t s, auto&& f, auto&& pad) {
            int64_t const r0 = sys_off[s];
            int32_t prev = 0;
            for (size_t q = 0; q < sip[s].size(); ++q) {
                int64_t const r = r0 + static_cast<int64_t>(q);
                int j = 0;
                for (int32_t k = prev; k < sip[s][q]; ++k, ++j)
                    f(r, j, six[s][k], cpx ? svc[s][k] : cd(svr[s][k], 0.0));
                for (; j < W; ++j) pad(r, j);
                prev = sip[s][q];
            }
        };
        with_vtype(vtype, [&](auto zc) {
            using Tc = decltype(zc);
            std::unique_ptr<Tc[]> val(new Tc[static_cast<size_t>(rows) * W * vs]);  // every slot is written below
            parallel_for(nsys, [&](int64_t s) {
                for_rows(
                    s,
                    [&](int64_t r, int j, int32_t c, cd const& h) {
                        col[r * W + j] = c;
                        Tc const hi = from_cd<Tc>(h);
                        val[(r * W + j) * vs] = hi;
                        if (vs == 2) val[(r * W + j) * vs + 1] = from_cd<Tc>(h - to_cd(hi));
                    },
                    [&](int64_t r, int j) {
                        col[r * W + j] = static_cast<int32_t>(r);
                        for (int q = 0; q < vs; ++q) val[(r * W + j) * vs + q] = Tc(0);
                    });
            });
            size_t const nval = static_cast<size_t>(rows) * W * vs;
            // 64 bytes of tail padding: bulk copies of a tile's entries round their size up to 16 bytes
            d_col.ensure(col.size() * sizeof(int32_t) + 64);
            d_val.ensure(nval * sizeof(Tc) + 64);
            upload_host(d_col.p, col.data(), col.size() * sizeof(int32_t));
            upload_host(d_val.p, val.get(), nval * sizeof(Tc));
            KPM_CUDA(cudaStreamSynchronize(stream));
        });
        // A complex H~ whose values are all real (e.g. a real lattice stored as complex so that
        // random-phase starters apply): the diagonal step can multiply by real values, two FMAs
        // per entry instead of four (same results: the imaginary parts are exact zeros)
        real_values = false;
        if (cpx) {
            std::vector<char> sys_real(nsys, 1);
            parallel_for(nsys, [&](int64_t s) {
                sys_real[s] = std::all_of(svc[s].begin(), svc[s].end(), [](cd const& h) { return h.imag() == 0.0; });
            });
            real_values = std::all_of(sys_real.begin(), sys_real.end(), [](char c) { return c != 0; });
            if (real_values) {
                auto upload = [&](auto zr) {
                    using Tr_ = decltype(zr);
                    int const rvs = std::is_same_v<Tr_, float> ? 2 : 1;  // FP32: (hi, lo) pairs
                    std::unique_ptr<Tr_[]> rv(new Tr_[static_cast<size_t>(rows) * W * rvs]);
                    parallel_for(nsys, [&](int64_t s) {
                        for_rows(
                            s,
                            [&](int64_t r, int j, int32_t, cd const& h) {
                                Tr_ const hi = static_cast<Tr_>(h.real());
                                rv[(r * W + j) * rvs] = hi;
                                if (rvs == 2) rv[(r * W + j) * rvs + 1] = static_cast<Tr_>(h.real() - static_cast<double>(hi));
                            },
                            [&](int64_t r, int j) {
                                for (int q = 0; q < rvs; ++q) rv[(r * W + j) * rvs + q] = Tr_(0);
                            });
                    });
                    size_t const n = static_cast<size_t>(rows) * W * rvs;
                    d_val_real.ensure(n * sizeof(Tr_) + 64);
                    upload_host(d_val_real.p, rv.get(), n * sizeof(Tr_));
                    KPM_CUDA(cudaStreamSynchronize(stream));
                };
                if (vtype == kpm::V_C64) upload(float{});
                else upload(double{});
            }
        }
        h_col = std::move(col);
        opt_nnz = total_nnz;
        d_map.ensure(sizeof(int32_t) * rows);
        upload_host(d_map.p, map.data(), sizeof(int32_t) * rows);
        d_sysoff.ensure(sizeof(int64_t) * (nsys + 1));
        KPM_CUDA(cudaMemcpyAsync(d_sysoff.p, sys_off.data(), sizeof(int64_t) * (nsys + 1), cudaMemcpyHostToDevice, stream));
        KPM_CUDA(cudaStreamSynchronize(stream));
        idx_src.clear();
        idx_dest.clear();
        for (auto i : src) idx_src.push_back(map[i]);
        for (auto i : dest) idx_dest.push_back(map[i]);
        // SliceMap offsets (OptimizedHamiltonian.cpp:5-18)
        auto find_offset = [&](std::vector<int32_t> const& idx) {
            int32_t const mx = *std::max_element(idx.begin(), idx.end());
            auto it = std::find_if(slices.begin(), slices.end(), [&](int32_t v) { return v > mx; });
            return static_cast<int64_t>(it - slices.begin());
        };
        src_offset = find_offset(idx_src);
        dest_offset = find_offset(idx_dest);
        opt_src = src;
        opt_dest = dest;
        opt_valid = true;
        pair_plans.clear();
        st.hamiltonian_time = now_s() - t0;
    }

    int64_t slice_index(int64_t n, int64_t M) const {  // SliceMap::index
        int64_t const last = static_cast<int64_t>(slices.size()) - 1;
        int64_t const mid = (M - 1 + dest_offset - src_offset) / 2;
        int64_t const mx = std::min(last, mid + src_offset);
        if (n < mid) return std::min(mx, n + src_offset);
        return std::min(mx, M - 1 - n + dest_offset);
    }
    int32_t optimal_size(int64_t n, int64_t M) const { return slices[slice_index(n, M)]; }

    // ---------------------------------------------------------------- batching
    struct Shape { int E, LPR, K, nbatch, rows_per_tile; };

    Shape pick_shape(int64_t nvec) const {
        int const vb = kpm::vtype_bytes(vtype);
        int const E16 = 16 / vb;
        int kmax = cfg.batch_width > 0 ? cfg.batch_width : 256 / vb;  // 256-byte rows by default
        Shape sh{1, 1, 1, 1, 0};
        if (nvec >= E16 * 2 && kmax >= E16 * 2) {
            int K = E16 * 2;
            while (K * 2 <= kmax && K * 2 <= nvec && K * 2 <= E16 * 32) K *= 2;
            sh.E = E16;
            sh.LPR = K / E16;
            sh.K = K;
        }
        if (cfg.batch_width == 1) sh = Shape{1, 1, 1, 1, 0};
        sh.nbatch = static_cast<int>((nvec + sh.K - 1) / sh.K);
        sh.rows_per_tile = (256 / sh.LPR) * 16;
        return sh;
    }

    // Autotuner: the launch options of a shape are picked by timing the diagonal kernel on
    // this engine's matrix, in its regular form (x1 <- H~ x0 - x1, the register footprint of
    // the recursion; the INIT form needs fewer registers and times differently). Only x1 and
    // the first accumulator slot change; the init step that follows overwrites x1 and the
    // caller clears the accumulators again. Cached per shape.
    // Choices are kept process-wide: a new engine on a matrix of the same size, width and
    // non-zero count (e.g. another disorder realisation) reuses them instead of timing again.
    struct TuneKey {
        int vtype, E, LPR, nbatch;
        int64_t rows, nnz;
        int W, staging, device;
        bool full_rows, real;
        int comp;
        bool operator==(TuneKey const& o) const {
            return vtype == o.vtype && E == o.E && LPR == o.LPR && nbatch == o.nbatch && rows == o.rows &&
                   nnz == o.nnz && W == o.W && staging == o.staging && device == o.device &&
                   full_rows == o.full_rows && real == o.real && comp == o.comp;
        }
    };
    TuneKey tune_key(Shape const& sh, bool full_rows) const {
        int dev = 0;
        cudaGetDevice(&dev);
        return TuneKey{vtype, sh.E, sh.LPR, sh.nbatch, rows, opt_nnz, W, cfg.staging, dev, full_rows, real_values,
                       compensated()};
    }
    struct Tuned { int rows_per_tile, unroll, E, LPR, prefetch = 0; };
    // FP32 real recursions: row sums compensated by an FMA per term (1: KPM_PREC_FP32P, and the
    // automatic precision of a float32 H) or by TwoSum (2: KPM_PREC_FP32X); 0 = chained FMAs
    int compensated() const {
        if (vtype != kpm::V_F32) return 0;
        if (cfg.precision == KPM_PREC_FP32X) return 2;
        return (cfg.precision == KPM_PREC_FP32P || cfg.precision == KPM_PREC_AUTO) ? 1 : 0;
    }
    // steps per launch chosen by timing the first steps of a recursion: 1, or 2 with a tile height
    struct FuseChoice { int steps, rows_per_tile; };
    template<class T>
    struct SharedCache {
        std::mutex m;
        std::vector<std::pair<TuneKey, T>> v;
        bool find(TuneKey const& k, T& out) {
            std::lock_guard<std::mutex> lock(m);
            for (auto const& e : v)
                if (e.first == k) { out = e.second; return true; }
            return false;
        }
        void put(TuneKey const& k, T const& t) {
            std::lock_guard<std::mutex> lock(m);
            v.push_back({k, t});
        }
    };
    static SharedCache<Tuned>& tuned() { static SharedCache<Tuned> c; return c; }
    static SharedCache<FuseChoice>& fuse_tuned() { static SharedCache<FuseChoice> c; return c; }

    static Shape timing_batches(Shape t) {
        t.nbatch = std::min(t.nbatch, 4);
        return t;
    }

    Tuned tune_diag(Shape sh, bool sys0, bool batch_outer, bool full_rows, kpm::DiagStep base) {
        // candidates are timed on up to four vector batches: a launch over several batches ranks
        // them differently from one (3D Anderson model, 4 batches of 64 vectors: staged entries
        // 3.79 against 3.32 ms per launch for per-row loads, though faster on one batch), and
        // more would make the timing cost scale with the batch count
        TuneKey const key = tune_key(sh, full_rows);
        {
            Tuned hit{};
            if (tuned().find(key, hit)) return hit;
        }
        Tuned best{(256 / sh.LPR) * 16, 1, sh.E, sh.LPR};
        // lane mappings of this K: the default (16 bytes per lane) and, when the row allows,
        // half the elements per lane over twice the lanes
        std::vector<std::pair<int, int>> maps{{sh.E, sh.LPR}};
        if (sh.E > 1 && kpm::diag_step_supported(vtype, sh.E / 2, sh.LPR * 2)) maps.push_back({sh.E / 2, sh.LPR * 2});
        {   // small problems (L2-resident, latency bound) want short tiles for parallelism,
            // large ones taller tiles for fewer flushes: timed either way
            double best_ms = 1e30;
            for (auto const& mp : maps)
                for (int unroll : {1, 2})
                    for (int rpt : {1, 2, 4, 8, 16, 32, 64}) {
                        if (rpt < 2 * unroll || cfg.staging == 2 || (compensated() == 2 && unroll != 1)) continue;
                        Shape t = sh;
                        t.E = mp.first;
                        t.LPR = mp.second;
                        t.rows_per_tile = (256 / t.LPR) * rpt;
                        base.E = t.E;
                        base.LPR = t.LPR;
                        base.num_tiles = build_tiles(timing_batches(t), sys0, batch_outer);
                        base.tiles = d_tiles.as<Tile>();
                        base.init = false;
                        base.unroll = unroll;
                        KPM_CUDA(kpm::launch_diag_step(base, stream));  // warm
                        KPM_CUDA(cudaEventRecord(ev0, stream));
                        for (int i = 0; i < 3; ++i) KPM_CUDA(kpm::launch_diag_step(base, stream));
                        KPM_CUDA(cudaEventRecord(ev1, stream));
                        KPM_CUDA(cudaEventSynchronize(ev1));
                        float ms = 0;
                        KPM_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
                        if (ms < best_ms) { best_ms = ms; best = Tuned{t.rows_per_tile, unroll, t.E, t.LPR}; }
                    }
            // the step with prefetched ELL entries (diag_pf_kernel): tiles of whole warp chunks
            // (8 warps x 16 rows), register allocation held to 4 blocks per SM or not
            base.unroll = 1;
            base.E = sh.E;
            base.LPR = sh.LPR;
            for (int pf : {3, 4})
                for (int chunks : {1, 2, 4, 8}) {
                    if (cfg.staging == 1 || compensated() == 2) break;
                    Shape t = sh;
                    t.rows_per_tile = 128 * chunks;
                    base.num_tiles = build_tiles(timing_batches(t), sys0, batch_outer);
                    base.tiles = d_tiles.as<Tile>();
                    base.init = false;
                    base.prefetch = pf;
                    cudaError_t const le = kpm::launch_diag_step(base, stream);  // warm
                    if (le == cudaErrorInvalidValue) {  // rows too wide for the shared-memory chunks
                        cudaGetLastError();
                        break;
                    }
                    KPM_CUDA(le);
                    KPM_CUDA(cudaEventRecord(ev0, stream));
                    for (int i = 0; i < 3; ++i) KPM_CUDA(kpm::launch_diag_step(base, stream));
                    KPM_CUDA(cudaEventRecord(ev1, stream));
                    KPM_CUDA(cudaEventSynchronize(ev1));
                    float ms = 0;
                    KPM_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
                    if (ms < best_ms) { best_ms = ms; best = Tuned{t.rows_per_tile, 1, sh.E, sh.LPR, pf}; }
                }
            base.prefetch = 0;
        }
        tuned().put(key, best);
        return best;
    }

    // Partition for the two-step kernel: tiles of `tpr` rows (per system, per batch), the
    // band of tiles each tile's rows touch (phase B of a tile waits for phase A of its band),
    // and the work queue in which B_t follows A_{max band hi over tiles <= t}.
    PairPlan* pair_plan(Shape const& sh, int tpr) {
        if (pair_key_nbatch != sh.nbatch || pair_key_lpr != sh.LPR || pair_key_rows != rows) {
            pair_plans.clear();
            pair_key_nbatch = sh.nbatch;
            pair_key_lpr = sh.LPR;
            pair_key_rows = rows;
        }
        for (auto& pp : pair_plans)
            if (pp->rows_per_tile == tpr) return pp.get();
        auto pp = std::make_unique<PairPlan>();
        pp->rows_per_tile = tpr;
        std::vector<Tile> tiles;
        std::vector<int64_t> base(nsys + 1, 0);  // row tiles before system s
        for (int s = 0; s < nsys; ++s) base[s + 1] = base[s] + (sys_rows(s) + tpr - 1) / tpr;
        // row-tile hull per row tile: tiles its rows read, widened by the tiles that read its rows
        // (equal for a Hermitian pattern; both are covered so that any pattern is safe)
        int64_t const RT = base[nsys];
        std::vector<int64_t> lo(RT), hi(RT);
        for (int64_t i = 0; i < RT; ++i) { lo[i] = i; hi[i] = i; }
        for (int s = 0; s < nsys; ++s)
            for (int64_t q = sys_off[s]; q < sys_off[s + 1]; ++q) {
                int64_t const tq = base[s] + (q - sys_off[s]) / tpr;
                for (int j = 0; j < W; ++j) {
                    int64_t const c = h_col[static_cast<size_t>(q) * W + j];
                    int64_t const tc = base[s] + (c - sys_off[s]) / tpr;
                    lo[tq] = std::min(lo[tq], tc); hi[tq] = std::max(hi[tq], tc);
                    lo[tc] = std::min(lo[tc], tq); hi[tc] = std::max(hi[tc], tq);
                }
            }
        std::vector<int32_t> band;
        for (int s = 0; s < nsys; ++s)
            for (int64_t r = sys_off[s]; r < sys_off[s + 1]; r += tpr) {
                int64_t const r1 = std::min(sys_off[s + 1], r + tpr);
                int64_t const rt = base[s] + (r - sys_off[s]) / tpr;
                for (int b = 0; b < sh.nbatch; ++b) {
                    tiles.push_back({static_cast<int32_t>(r), static_cast<int32_t>(r1), s, b});
                    band.push_back(static_cast<int32_t>(lo[rt] * sh.nbatch + b));
                    band.push_back(static_cast<int32_t>(hi[rt] * sh.nbatch + b));
                }
            }
        int const T = static_cast<int>(tiles.size());
        std::vector<int32_t> items;
        items.reserve(2 * T);
        // B_t is queued `lag` phase-A items after the last A it needs, so that those are
        // usually finished when B_t is handed out (about the number of blocks in flight)
        int dev = 0, sms = 152;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        int32_t const lag = 2 * sms;
        int32_t hstar = -1;
        std::vector<int32_t> hs(T);
        for (int t = 0; t < T; ++t) {
            hstar = std::max(hstar, band[2 * t + 1]);
            hs[t] = std::min<int32_t>(T - 1, hstar + lag);
        }
        int pb = 0;
        for (int k = 0; k < T; ++k) {
            items.push_back(2 * k);
            while (pb < T && hs[pb] <= k) items.push_back(2 * pb++ + 1);
        }
        while (pb < T) items.push_back(2 * pb++ + 1);
        pp->num_tiles = T;
        pp->d_tiles.ensure(sizeof(Tile) * T);
        pp->d_items.ensure(sizeof(int32_t) * 2 * T);
        pp->d_band.ensure(sizeof(int32_t) * 2 * T);
        pp->d_flags.ensure(sizeof(int32_t) * T);
        KPM_CUDA(cudaMemcpyAsync(pp->d_tiles.p, tiles.data(), sizeof(Tile) * T, cudaMemcpyHostToDevice, stream));
        KPM_CUDA(cudaMemcpyAsync(pp->d_items.p, items.data(), sizeof(int32_t) * 2 * T, cudaMemcpyHostToDevice, stream));
        KPM_CUDA(cudaMemcpyAsync(pp->d_band.p, band.data(), sizeof(int32_t) * 2 * T, cudaMemcpyHostToDevice, stream));
        KPM_CUDA(cudaMemsetAsync(pp->d_flags.p, 0, sizeof(int32_t) * T, stream));
        KPM_CUDA(cudaStreamSynchronize(stream));
        pair_plans.push_back(std::move(pp));
        return pair_plans.back().get();
    }

    int next_seq() {
        if (pair_seq >= (1 << 30)) {  // restart the sequence: clear every plan's flags
            for (auto& pp : pair_plans)
                KPM_CUDA(cudaMemsetAsync(pp->d_flags.p, 0, sizeof(int32_t) * pp->num_tiles, stream));
            pair_seq = 0;
        }
        return ++pair_seq;
    }

    // Tiles of (rows, system, batch). Batch innermost ([tile][batch]) lets a shrinking row
    // limit cut the list at a tile boundary; batch outermost makes the persistent blocks sweep
    // one batch at a time, so the gathered x rows that must stay in L2 belong to one batch
    // (3D lattices: neighbours lie a whole BFS shell away).
    int build_tiles(Shape const& sh, bool sys0_only, bool batch_outer = false) {
        std::vector<Tile> tiles;
        int const ns = sys0_only ? 1 : nsys;
        auto add = [&](int s, int64_t r, int b) {
            tiles.push_back({static_cast<int32_t>(r), static_cast<int32_t>(std::min(sys_off[s + 1], r + sh.rows_per_tile)),
                             s, b});
        };
        if (batch_outer) {
            for (int b = 0; b < sh.nbatch; ++b)
                for (int s = 0; s < ns; ++s)
                    for (int64_t r = sys_off[s]; r < sys_off[s + 1]; r += sh.rows_per_tile) add(s, r, b);
        } else {
            for (int s = 0; s < ns; ++s)
                for (int64_t r = sys_off[s]; r < sys_off[s + 1]; r += sh.rows_per_tile)
                    for (int b = 0; b < sh.nbatch; ++b) add(s, r, b);
        }
        d_tiles.ensure(sizeof(Tile) * tiles.size());
        KPM_CUDA(cudaMemcpyAsync(d_tiles.p, tiles.data(), sizeof(Tile) * tiles.size(), cudaMemcpyHostToDevice, stream));
        return static_cast<int>(tiles.size());
    }

    // ---------------------------------------------------------------- diagonal recursion
    // Starters: kind 0 = host/device array [s][v][i] original order, kind 1 = unit vectors at
    // reordered positions `units` (system 0). Per-vector moments land in d_mu as
    // [s][v][M] complex double. `opt_rows` applies the optimal-size row limit (system 0).
    void run_diag(int64_t M, int64_t nvec, void const* starters, bool on_device, std::vector<int32_t> const* units,
                  bool opt_rows, bool units_per_system = false) {
        if (M < 2 || (M - 2) % 4 != 0) fail(KPM_ERR_VALUE, "num_moments must satisfy (M - 2) % 4 == 0");
        if (nvec < 1) fail(KPM_ERR_VALUE, "num_vectors must be >= 1");
        Shape sh = pick_shape(nvec);
        int const vb = kpm::vtype_bytes(vtype);
        int const NV = kpm::vtype_nv(vtype);
        // units: nvec unit vectors in system 0, or (units_per_system) one vector holding a
        // unit entry in every system, at units[s]
        bool const sys0 = units != nullptr && !units_per_system;
        if (units_per_system && (nvec != 1 || !units || static_cast<int>(units->size()) != nsys))
            fail(KPM_ERR_VALUE, "one unit position per system and one vector");
        int const ns = sys0 ? 1 : nsys;
        int64_t const bstride = rows * sh.K;
        size_t const vbytes = static_cast<size_t>(bstride) * sh.nbatch * vb;
        d_x0.ensure(vbytes);
        d_x1.ensure(vbytes);
        int64_t const half = M / 2;
        size_t const step_acc = static_cast<size_t>(ns) * sh.nbatch * sh.K * NV;
        d_acc.ensure(sizeof(double) * step_acc * half);
        d_mu.ensure(sizeof(double) * 2 * ns * nvec * M);
        // tiles batch-outermost (L2 then holds one batch's gather window); with a shrinking row
        // limit the tiles beyond it are launched and do nothing (the kernel clips rows)
        bool const batch_outer = true;
        bool const full_rows = !opt_rows;  // the TMA and cp.async kernels do not clip rows
        int ntiles = build_tiles(sh, sys0, batch_outer);

        // r0 = the starters, in the layout of shape `ls`
        void const* starter_src = nullptr;
        auto load_starters = [&](Shape const& ls) {
            KPM_CUDA(cudaMemsetAsync(d_x0.p, 0, vbytes, stream));
            if (units) {
                d_pos.ensure(sizeof(int32_t) * units->size());
                KPM_CUDA(cudaMemcpyAsync(d_pos.p, units->data(), sizeof(int32_t) * units->size(), cudaMemcpyHostToDevice, stream));
                if (units_per_system)
                    for (int s = 0; s < nsys; ++s)
                        KPM_CUDA(kpm::launch_set_units(vtype, d_x0.p, d_pos.as<int32_t>() + s, 1, ls.K, rows, stream));
                else
                    KPM_CUDA(kpm::launch_set_units(vtype, d_x0.p, d_pos.as<int32_t>(), nvec, ls.K, rows, stream));
            } else {
                // starters are in the Hamiltonian's scalar type; the scatter converts them. Host starters:
                // where the GPU reads host memory through the host page tables (Grace), the scatter
                // kernel reads them in place; elsewhere they are staged in device memory first
                if (starter_src == nullptr) {
                    size_t const in_bytes = static_cast<size_t>(nvec) * rows * scalar_bytes(stype);
                    starter_src = on_device ? starters : device_view(starters, in_bytes);
                }
                KPM_CUDA(kpm::launch_scatter_starters(stype, vtype, starter_src, d_x0.p, d_map.as<int32_t>(),
                                                      d_sysoff.as<int64_t>(), nsys, nvec, ls.K, ls.nbatch, rows, stream));
            }
        };
        KPM_CUDA(cudaEventRecord(ev_u0, stream));
        load_starters(sh);
        KPM_CUDA(cudaEventRecord(ev_u1, stream));
        kpm::DiagStep a{};
        a.vtype = vtype;
        a.E = sh.E;
        a.LPR = sh.LPR;
        a.col = d_col.as<int32_t>();
        a.val = real_values ? d_val_real.p : d_val.p;
        a.real_matrix = real_values;
        a.W = W;
        a.batch_stride = bstride;
        a.tiles = d_tiles.as<Tile>();
        a.num_tiles = ntiles;
        a.nbatch = sh.nbatch;
        a.row_limit = static_cast<int32_t>(rows);
        a.x = d_x0.p;
        a.y = d_x1.p;
        a.acc = d_acc.as<double>();
        bool alt_map = false;  // a thinner lane mapping: single-step launches only
        a.compensated = compensated();
        d_pair_error.ensure(sizeof(int));
        KPM_CUDA(cudaMemsetAsync(d_pair_error.p, 0, sizeof(int), stream));
        if (cfg.tile_rows > 0) {
            sh.rows_per_tile = cfg.tile_rows;
            if (cfg.staging == 2 && kpm::diag_pf_supported(vtype, W, sh.LPR)) a.prefetch = 4;
        } else {
            Tuned const tu = tune_diag(sh, sys0, batch_outer, full_rows, a);
            sh.rows_per_tile = tu.rows_per_tile;
            a.unroll = tu.unroll;
            a.prefetch = tu.prefetch;
            alt_map = tu.E != sh.E;
            if (alt_map && cfg.fuse_steps == 2 && !opt_rows) {  // two-step launches asked for: default kernel
                alt_map = false;
                sh.rows_per_tile = (256 / sh.LPR) * 16;
                a.unroll = 1;
                a.prefetch = 0;
            } else {
                sh.E = tu.E;
                sh.LPR = tu.LPR;
            }
            a.E = sh.E;
            a.LPR = sh.LPR;
        }
        ntiles = build_tiles(sh, sys0, batch_outer);
        a.tiles = d_tiles.as<Tile>();
        a.num_tiles = ntiles;
        KPM_CUDA(cudaEventRecord(ev0, stream));
        void* r0 = d_x0.p;
        void* r1 = d_x1.p;
        int64_t n = 2;
        // r1 = H~ r0 / 2 with mu0, mu1 sums
        auto first_step = [&]() {
            KPM_CUDA(cudaMemsetAsync(d_acc.p, 0, sizeof(double) * step_acc * half, stream));
            a.x = d_x0.p;
            a.y = d_x1.p;
            a.acc = d_acc.as<double>();
            a.init = true;
            KPM_CUDA(kpm::launch_diag_step(a, stream));
            a.init = false;
            r0 = d_x0.p;
            r1 = d_x1.p;
            n = 2;
        };
        first_step();
        auto single_step = [&]() {
            a.x = r1;
            a.y = r0;
            a.acc = d_acc.as<double>() + step_acc * (n - 1);
            if (opt_rows) {
                int32_t const lim = optimal_size(n, M);
                a.row_limit = lim;
                // one batch: the tiles that start below the limit are a prefix of the list;
                // several (batch-outer order): all are launched, rows beyond the limit are skipped
                if (sh.nbatch == 1) {
                    int64_t const t = (lim + sh.rows_per_tile - 1) / sh.rows_per_tile;
                    a.num_tiles = static_cast<int>(std::min<int64_t>(ntiles, t));
                }
            }
            KPM_CUDA(kpm::launch_diag_step(a, stream));
            std::swap(r0, r1);
            ++n;
        };
        // two steps per launch: P = r0 (T_{n-2} -> T_n), Q = r1 (T_{n-1} -> T_{n+1}); the
        // roles are unchanged after the pair, so no swap
        int64_t const max_pairs = std::max<int64_t>(1, half / 2);
        d_pair_counters.ensure(sizeof(unsigned) * max_pairs);
        KPM_CUDA(cudaMemsetAsync(d_pair_counters.p, 0, sizeof(unsigned) * max_pairs, stream));
        int64_t pair_index = 0;
        auto pair_step = [&](PairPlan* pp) {
            kpm::DiagPair q{};
            q.vtype = vtype;
            q.E = sh.E;
            q.LPR = sh.LPR;
            q.col = d_col.as<int32_t>();
            q.val = d_val.p;
            q.W = W;
            q.P = r0;
            q.Q = r1;
            q.batch_stride = bstride;
            q.tiles = pp->d_tiles.as<Tile>();
            q.items = pp->d_items.as<int32_t>();
            q.band = pp->d_band.as<int32_t>();
            q.num_tiles = pp->num_tiles;
            q.nbatch = sh.nbatch;
            q.flags = pp->d_flags.as<int>();
            q.seq = next_seq();
            q.counter = d_pair_counters.as<unsigned>() + pair_index++;
            q.accA = d_acc.as<double>() + step_acc * (n - 1);
            q.accB = d_acc.as<double>() + step_acc * n;
            q.error = d_pair_error.as<int>();
            q.spin_limit = 1 << 24;  // x ~64 ns sleeps: gives up after about a second
            KPM_CUDA(kpm::launch_diag_pair(q, stream));
            n += 2;
        };
        int const rpp = 256 / sh.LPR;
        bool const can_pair = !opt_rows && cfg.fuse_steps != 1 && !alt_map && !a.compensated;
        FuseChoice choice{1, 0};
        TuneKey const fkey = tune_key(sh, full_rows);
        bool have_choice = fuse_tuned().find(fkey, choice);
        if (can_pair && cfg.fuse_steps == 2 && !have_choice) {
            choice = FuseChoice{2, cfg.tile_rows > 0 ? cfg.tile_rows : rpp * 8};
            have_choice = true;
        }
        if (can_pair && !have_choice) {
            // time each candidate on four steps of this recursion, keep the fastest, then start
            // the recursion over with it
            std::vector<FuseChoice> cands{{1, 0}};
            for (int rpt : {4, 8, 16, 32}) cands.push_back({2, rpp * rpt});
            double best = 1e30;
            if (half - 1 >= 4 * static_cast<int64_t>(cands.size()) + 2) {
                for (auto const& c : cands) {
                    PairPlan* pp = c.steps == 2 ? pair_plan(sh, c.rows_per_tile) : nullptr;
                    KPM_CUDA(cudaEventRecord(ev_t0, stream));
                    if (pp) { pair_step(pp); pair_step(pp); }
                    else for (int k = 0; k < 4; ++k) single_step();
                    KPM_CUDA(cudaEventRecord(ev_t1, stream));
                    KPM_CUDA(cudaEventSynchronize(ev_t1));
                    float ms = 0;
                    KPM_CUDA(cudaEventElapsedTime(&ms, ev_t0, ev_t1));
                    if (ms < best) { best = ms; choice = c; }
                }
                fuse_tuned().put(fkey, choice);
                // the candidates' partial moment sums round differently (FP32 partials over
                // different tiles): start over with the chosen one, so that this call's moments
                // are those of every later call
                load_starters(sh);
                first_step();
                KPM_CUDA(cudaMemsetAsync(d_pair_counters.p, 0, sizeof(unsigned) * max_pairs, stream));
                pair_index = 0;
            } else {
                choice = FuseChoice{1, 0};
            }
        }
        if (cfg.fuse_steps == 2 && can_pair && choice.steps != 2)
            choice = FuseChoice{2, cfg.tile_rows > 0 ? cfg.tile_rows : rpp * 8};
        if (choice.steps == 2 && can_pair) {
            PairPlan* pp = pair_plan(sh, choice.rows_per_tile);
            while (n + 1 <= half) pair_step(pp);
        }
        int progress_segments = 0;
        if (progress_total > 0 && progress_fn && n <= half) {
            // reported progress: the remaining steps in segments, each followed by an event that
            // the host waits on below (the launches are all queued first, so the GPU never idles)
            int64_t const n0 = n, left = half - n + 1;
            for (int k = 0; k < kProgressSegments; ++k) {
                if (!progress_ev[k]) KPM_CUDA(cudaEventCreateWithFlags(&progress_ev[k], cudaEventDisableTiming));
                int64_t const stop = n0 + left * (k + 1) / kProgressSegments;
                while (n < stop) single_step();
                KPM_CUDA(cudaEventRecord(progress_ev[k], stream));
            }
            progress_segments = kProgressSegments;
        }
        if (n == 2 && half >= 3 && !opt_rows) {
            // steady state (no tuning steps ran in this call): replay the captured recursion
            RecursionGraphKey key{};
            std::memset(&key, 0, sizeof key);  // padding bytes take part in the comparison
            key.x0 = d_x0.p;
            key.x1 = d_x1.p;
            key.acc = d_acc.p;
            key.tiles = a.tiles;
            key.col = a.col;
            key.val = a.val;
            key.half = half;
            key.bstride = bstride;
            key.step_acc = static_cast<int64_t>(step_acc);
            key.ntiles = a.num_tiles;
            key.vtype = vtype;
            key.E = sh.E;
            key.LPR = sh.LPR;
            key.nbatch = sh.nbatch;
            key.unroll = a.unroll;
            key.W = W;
            key.row_limit = a.row_limit;
            key.real_matrix = a.real_matrix;
            key.prefetch = a.prefetch;
            if (graph_exec == nullptr || !(key == graph_key)) {
                drop_graph();
                KPM_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
                cudaGraph_t g = nullptr;
                try {
                    while (n <= half) single_step();
                } catch (...) {
                    cudaStreamEndCapture(stream, &g);
                    if (g) cudaGraphDestroy(g);
                    throw;
                }
                KPM_CUDA(cudaStreamEndCapture(stream, &g));
                cudaError_t const ie = cudaGraphInstantiate(&graph_exec, g, 0);
                cudaGraphDestroy(g);
                if (ie != cudaSuccess) {
                    graph_exec = nullptr;
                    KPM_CUDA(ie);
                }
                std::memcpy(&graph_key, &key, sizeof key);  // padding included
            } else {
                n = half + 1;
            }
            KPM_CUDA(cudaGraphLaunch(graph_exec, stream));
        }
        while (n <= half) single_step();
        last_fuse = choice.steps;
        last_unroll = a.unroll;
        last_prefetch = a.prefetch;
        KPM_CUDA(cudaEventRecord(ev1, stream));
        KPM_CUDA(kpm::launch_collect_diag(vtype, d_acc.as<double>(), ns, sh.nbatch, sh.K, half, M, nvec, false,
                                          d_mu.as<double>(), stream));
        int pair_err = 0;
        KPM_CUDA(cudaMemcpyAsync(&pair_err, d_pair_error.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
        for (int k = 0; k < progress_segments; ++k) {
            KPM_CUDA(cudaEventSynchronize(progress_ev[k]));
            progress(progress_total * (k + 1) / progress_segments - progress_total * k / progress_segments);
        }
        KPM_CUDA(cudaStreamSynchronize(stream));
        if (pair_err)
            fail(KPM_ERR_TIMEOUT, "a two-step recursion launch gave up waiting for a neighbouring tile; results "
                                  "discarded");
        float ms = 0;
        KPM_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
        st.moments_time = ms * 1e-3;
        float ums = 0;
        KPM_CUDA(cudaEventElapsedTime(&ums, ev_u0, ev_u1));
        last_upload_time = ums * 1e-3;
        last_shape = sh;
    }
    Shape last_shape{};
    int last_fuse = 1;
    int last_unroll = 1;
    int last_prefetch = 0;
    double last_upload_time = 0;
    cudaEvent_t ev_t0 = nullptr, ev_t1 = nullptr;
    cudaEvent_t ev_u0 = nullptr, ev_u1 = nullptr;  // starter upload + scatter of the last diagonal call

    void reset_stats(int64_t M, bool diagonal, bool opt, double multiplier, int64_t active_rows_nnz_rows) {
        (void)active_rows_nnz_rows;
        st.num_moments = M;
        st.gemm_time = 0;
        st.multiplier = multiplier;
        int64_t const ell_nnz = rows * W;
        st.uses_full_system = static_cast<int32_t>(static_cast<int64_t>(slices.size()) < M / 2);
        int64_t nnz = M * ell_nnz, vec = M * rows;
        int64_t onnz = nnz, ovec = vec;
        if (opt) {
            onnz = 0;
            ovec = 0;
            for (int64_t n = 0; n < M; ++n) {
                int64_t const sz = optimal_size(n, M);
                onnz += sz * W;
                ovec += sz;
            }
        }
        if (diagonal) { nnz /= 2; onnz /= 2; vec /= 2; ovec /= 2; }
        st.nnz = nnz;
        st.opt_nnz = onnz;
        st.vec = vec;
        st.opt_vec = ovec;
        st.matrix_memory = static_cast<int64_t>(rows) * W * (kpm::vtype_vs(vtype) * kpm::vtype_bytes(vtype) + 4);
        st.vector_memory = static_cast<int64_t>(rows) * kpm::vtype_bytes(vtype);
    }
    void finish_stats() {
        st.eps = st.moments_time > 0 ? st.multiplier * st.opt_nnz / st.moments_time : 0.0;
        st.steps_per_launch = last_fuse;
        st.elems_per_lane = last_shape.E;
        st.lanes_per_row = last_shape.LPR;
        st.staged_rows = 0;
        st.prefetch = last_prefetch;
        st.gather_rows = 0;
        st.tile_rows = last_shape.rows_per_tile;
        st.unroll = last_unroll;
        st.upload_time = last_upload_time;
    }

    // ---------------------------------------------------------------- reconstruction
    void spectral(double const* d_moments_cd, int64_t M, int cols, double const* energy, int64_t ne, ScaleAB sc,
                  double* out_host) {
        d_energy.ensure(sizeof(double) * std::max<int64_t>(ne, 1));
        d_out.ensure(sizeof(double) * 2 * std::max<int64_t>(ne * cols, 1));
        KPM_CUDA(cudaMemcpyAsync(d_energy.p, energy, sizeof(double) * ne, cudaMemcpyHostToDevice, stream));
        KPM_CUDA(kpm::launch_spectral_density(d_moments_cd, M, cols, d_energy.as<double>(), static_cast<int>(ne),
                                              sc.a, sc.b, d_out.as<double>(), stream));
        KPM_CUDA(cudaMemcpyAsync(out_host, d_out.p, sizeof(double) * ne * cols, cudaMemcpyDeviceToHost, stream));
        KPM_CUDA(cudaStreamSynchronize(stream));
    }

    // damp per-column complex moments in place on the device copy (host round trip is tiny)
    void damp_device(double* d_moments_cd, int64_t M, int64_t cols, int64_t stride_M) {
        std::vector<double> h(static_cast<size_t>(2 * cols * stride_M));
        KPM_CUDA(cudaMemcpyAsync(h.data(), d_moments_cd, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, stream));
        KPM_CUDA(cudaStreamSynchronize(stream));
        auto g = damping(cfg.kernel, cfg.kernel_param, M);
        std::vector<double> o(static_cast<size_t>(2 * cols * M));
        for (int64_t c = 0; c < cols; ++c)
            for (int64_t n = 0; n < M; ++n) {
                o[2 * (c * M + n)] = h[2 * (c * stride_M + n)] * g[n];
                o[2 * (c * M + n) + 1] = h[2 * (c * stride_M + n) + 1] * g[n];
            }
        KPM_CUDA(cudaMemcpyAsync(d_moments_cd, o.data(), sizeof(double) * o.size(), cudaMemcpyHostToDevice, stream));
    }
};

namespace kpm {
void set_last_error(std::string const& msg) { g_last_error = msg; }
}  // namespace kpm

// ====================================================================== C ABI
extern "C" {

const char* kpm_last_error(void) { return g_last_error.c_str(); }

void kpm_config_default(kpm_config* c) {
    if (!c) return;
    c->min_energy = 0;
    c->max_energy = 0;
    c->kernel = KPM_KERNEL_JACKSON;
    c->kernel_param = 4.0;
    c->matrix_format = KPM_FORMAT_ELL;
    c->optimal_size = 1;
    c->interleaved = 1;
    c->lanczos_precision = 0.002;
    c->precision = KPM_PREC_AUTO;
    c->batch_width = 0;
    c->tile_rows = 0;
    c->fuse_steps = 0;
    c->staging = 0;
    c->num_threads = 0;
}

int kpm_create(int32_t scalar_type, int64_t rows, const int32_t* indptr, const int32_t* indices, const void* values,
               int32_t num_systems, const int64_t* system_offsets, const kpm_config* cfg, kpm_engine** out) {
    return guarded([&] {
        if (!out) fail(KPM_ERR_VALUE, "null output handle");
        *out = nullptr;
        auto e = std::make_unique<kpm_engine>();
        if (cfg) e->cfg = *cfg; else kpm_config_default(&e->cfg);
        // Config holds the energy range as float (kpm/Config.hpp:24-25)
        e->cfg.min_energy = static_cast<float>(e->cfg.min_energy);
        e->cfg.max_energy = static_cast<float>(e->cfg.max_energy);
        if (e->cfg.min_energy > e->cfg.max_energy)
            fail(KPM_ERR_VALUE, "KPM: Invalid energy range specified (min > max).");
        if (e->cfg.kernel == KPM_KERNEL_LORENTZ && e->cfg.kernel_param <= 0)
            fail(KPM_ERR_VALUE, "Lorentz kernel: lambda must be positive.");
        if (e->cfg.precision < KPM_PREC_AUTO || e->cfg.precision > KPM_PREC_FP32P)
            fail(KPM_ERR_VALUE, "unknown precision mode");
        if (e->cfg.fuse_steps < 0 || e->cfg.fuse_steps > 2) fail(KPM_ERR_VALUE, "fuse_steps must be 0, 1 or 2");
        if (e->cfg.staging < 0 || e->cfg.staging > 2) fail(KPM_ERR_VALUE, "staging must be 0, 1 or 2");
        e->set_h(scalar_type, rows, indptr, indices, values, num_systems, system_offsets);
        *out = e.release();
    });
}

int kpm_create_batch(kpm_engine* const* engines, int32_t num_engines, const kpm_config* cfg, kpm_engine** out) {
    return guarded([&] {
        if (!out) fail(KPM_ERR_VALUE, "null output handle");
        *out = nullptr;
        if (!engines || num_engines < 1) fail(KPM_ERR_VALUE, "no engines to batch");
        int64_t rows = 0, nnz = 0;
        for (int32_t i = 0; i < num_engines; ++i) {
            kpm_engine const* src = engines[i];
            if (!src) fail(KPM_ERR_VALUE, "null engine in the batch");
            if (src->nsys != 1) fail(KPM_ERR_VALUE, "batched engines must hold one system each");
            if (src->stype != engines[0]->stype) fail(KPM_ERR_VALUE, "batched engines must share the scalar type");
            rows += src->rows;
            nnz += src->indptr[src->rows];
        }
        if (rows > std::numeric_limits<int32_t>::max() || nnz > std::numeric_limits<int32_t>::max())
            fail(KPM_ERR_VALUE, "the batch exceeds int32 indices");
        auto e = std::make_unique<kpm_engine>();
        if (cfg) e->cfg = *cfg; else kpm_config_default(&e->cfg);
        e->cfg.min_energy = static_cast<float>(e->cfg.min_energy);
        e->cfg.max_energy = static_cast<float>(e->cfg.max_energy);
        if (e->cfg.min_energy > e->cfg.max_energy)
            fail(KPM_ERR_VALUE, "KPM: Invalid energy range specified (min > max).");
        if (e->cfg.kernel == KPM_KERNEL_LORENTZ && e->cfg.kernel_param <= 0)
            fail(KPM_ERR_VALUE, "Lorentz kernel: lambda must be positive.");
        if (e->cfg.precision < KPM_PREC_AUTO || e->cfg.precision > KPM_PREC_FP32P)
            fail(KPM_ERR_VALUE, "unknown precision mode");
        if (e->cfg.fuse_steps < 0 || e->cfg.fuse_steps > 2) fail(KPM_ERR_VALUE, "fuse_steps must be 0, 1 or 2");
        if (e->cfg.staging < 0 || e->cfg.staging > 2) fail(KPM_ERR_VALUE, "staging must be 0, 1 or 2");
        // the members' CSR matrices were checked when their engines were made: concatenate them
        // (columns shifted into their block), each member's copy in parallel
        int const st = engines[0]->stype;
        size_t const sb = static_cast<size_t>(scalar_bytes(st));
        std::vector<int64_t> row_off(num_engines + 1, 0), nz_off(num_engines + 1, 0);
        for (int32_t i = 0; i < num_engines; ++i) {
            row_off[i + 1] = row_off[i] + engines[i]->rows;
            nz_off[i + 1] = nz_off[i] + engines[i]->indptr[engines[i]->rows];
        }
        e->stype = st;
        e->rows = rows;
        e->nsys = num_engines;
        e->sys_off = row_off;
        e->indptr.resize(rows + 1);
        e->indices.resize(nnz);
        e->values.resize(static_cast<size_t>(nnz) * sb);
        e->indptr[0] = 0;
        parallel_for(num_engines, [&](int64_t i) {
            kpm_engine const* src = engines[i];
            int32_t const r0 = static_cast<int32_t>(row_off[i]), z0 = static_cast<int32_t>(nz_off[i]);
            for (int64_t r = 0; r < src->rows; ++r) e->indptr[r0 + r + 1] = z0 + src->indptr[r + 1];
            int64_t const n = src->indptr[src->rows];
            for (int64_t k = 0; k < n; ++k) e->indices[z0 + k] = r0 + src->indices[k];
            std::memcpy(e->values.data() + static_cast<size_t>(z0) * sb, src->values.data(), static_cast<size_t>(n) * sb);
        });
        e->sys.assign(num_engines, kpm_engine::Sys{});
        for (int32_t i = 0; i < num_engines; ++i) {
            if (e->cfg.min_energy != e->cfg.max_energy) {
                e->sys[i].have_bounds = true;
                e->sys[i].emin = e->cfg.min_energy;
                e->sys[i].emax = e->cfg.max_energy;
            } else if (engines[i]->sys[0].have_bounds && engines[i]->cfg.min_energy == engines[i]->cfg.max_energy &&
                       engines[i]->cfg.lanczos_precision == e->cfg.lanczos_precision) {
                e->sys[i] = engines[i]->sys[0];  // Lanczos bounds the member already found
            }
        }
        bool const dbl = e->cfg.precision == KPM_PREC_FP64 ||
                         (e->cfg.precision == KPM_PREC_AUTO && (st == KPM_F64 || st == KPM_C128));
        bool const cpx = scalar_complex(st);
        e->vtype = cpx ? (dbl ? kpm::V_C128 : kpm::V_C64) : (dbl ? kpm::V_F64 : kpm::V_F32);
        *out = e.release();
    });
}

int kpm_destroy(kpm_engine* engine) {
    return guarded([&] {
        if (engine) {
            if (engine->stream) cudaStreamSynchronize(engine->stream);
            delete engine;
        }
    });
}

int kpm_set_hamiltonian(kpm_engine* e, int32_t scalar_type, int64_t rows, const int32_t* indptr,
                        const int32_t* indices, const void* values, int32_t num_systems,
                        const int64_t* system_offsets) {
    return guarded([&] {
        if (!e) fail(KPM_ERR_VALUE, "null engine");
        HostThreads host_threads(e->cfg.num_threads);
        e->set_h(scalar_type, rows, indptr, indices, values, num_systems, system_offsets);
    });
}

int kpm_energy_bounds(kpm_engine* e, int32_t system, double* mn, double* mx, int32_t* loops) {
    return guarded([&] {
        if (!e) fail(KPM_ERR_VALUE, "null engine");
        HostThreads host_threads(e->cfg.num_threads);
        if (system < 0 || system >= e->nsys) fail(KPM_ERR_VALUE, "system index out of range");
        e->compute_bounds();
        if (mn) *mn = e->sys[system].emin;
        if (mx) *mx = e->sys[system].emax;
        if (loops) *loops = e->sys[system].loops;
    });
}

int kpm_scaling_factors(kpm_engine* e, int32_t system, double* a, double* b) {
    return guarded([&] {
        if (!e) fail(KPM_ERR_VALUE, "null engine");
        HostThreads host_threads(e->cfg.num_threads);
        if (system < 0 || system >= e->nsys) fail(KPM_ERR_VALUE, "system index out of range");
        auto const s = e->scale(system);
        if (a) *a = s.a;
        if (b) *b = s.b;
    });
}

int kpm_moments_diag(kpm_engine* e, int64_t num_moments, int64_t num_vectors, const void* starters,
                     int32_t starters_on_device, int32_t average, double* out, int64_t* num_moments_out) {
    return guarded([&] {
        if (!e) fail(KPM_ERR_VALUE, "null engine");
        HostThreads host_threads(e->cfg.num_threads);
        if (!starters || !out) fail(KPM_ERR_VALUE, "null starters or output");
        int64_t const M = round_moments(num_moments);
        double const t0 = now_s();
        e->optimize({0}, {0});
        e->run_diag(M, num_vectors, starters, starters_on_device != 0, nullptr, false);
        e->reset_stats(M, true, false, static_cast<double>(num_vectors) * e->nsys, 0);
        int64_t const cols = average ? e->nsys : e->nsys * num_vectors;
        if (average) {
            e->d_mu_avg.ensure(sizeof(double) * 2 * e->nsys * M);
            KPM_CUDA(kpm::launch_average(e->d_mu.as<double>(), e->nsys, num_vectors, M, e->d_mu_avg.as<double>(), e->stream));
            KPM_CUDA(cudaMemcpyAsync(out, e->d_mu_avg.p, sizeof(double) * 2 * cols * M, cudaMemcpyDeviceToHost, e->stream));
        } else {
            KPM_CUDA(cudaMemcpyAsync(out, e->d_mu.p, sizeof(double) * 2 * cols * M, cudaMemcpyDeviceToHost, e->stream));
        }
        KPM_CUDA(cudaStreamSynchronize(e->stream));
        e->finish_stats();
        e->calc_time = now_s() - t0;
        if (num_moments_out) *num_moments_out = M;
    });
}

int kpm_calc_dos(kpm_engine* e, const double* energy, int64_t ne, double broadening, int64_t num_random, double* out) {
    return guarded([&] {
        if (!e) fail(KPM_ERR_VALUE, "null engine");
        HostThreads host_threads(e->cfg.num_threads);
        if (num_random < 1) fail(KPM_ERR_VALUE, "num_random must be >= 1");
        if (ne > 0 && (!energy || !out)) fail(KPM_ERR_VALUE, "null energy or output");
        double const t0 = now_s();
        e->compute_bounds();
        std::vector<int64_t> Ms(e->nsys);
        int64_t Mmax = 2;
        for (int s = 0; s < e->nsys; ++s) {
            Ms[s] = required_moments(e->cfg.kernel, e->cfg.kernel_param, broadening / e->scale(s).a);
            Mmax = std::max(Mmax, Ms[s]);
        }
        e->optimize({0}, {0});
        // the reference's random starters: one default-seeded mt19937 per system (Starter.cpp:48-84),
        // in the Hamiltonian's scalar type
        // kept by the engine between calls: the GPU reads it in place, and pages it has seen
        // before are cheaper to read again
        std::vector<unsigned char>& st = e->h_starters;
        st.resize(static_cast<size_t>(num_random) * e->rows * scalar_bytes(e->stype));
        with_scalar(e->stype, [&](auto zi) {
            using Tin = decltype(zi);
            using R = real_of<Tin>;
            auto* o = reinterpret_cast<Tin*>(st.data());
            // each system's generator draws in the reference's order; systems are independent
            // and run in parallel, and the phases of complex starters are taken in parallel after
            std::vector<R> draws(is_cplx_v<Tin> ? st.size() / sizeof(Tin) : 0);
            parallel_for(e->nsys, [&](int64_t s) {
                int64_t const n = e->sys_rows(s);
                int64_t const base = e->sys_off[s] * num_random;
                std::mt19937 gen;
                std::uniform_real_distribution<R> dist;
                for (int64_t q = 0; q < num_random * n; ++q) {
                    if constexpr (is_cplx_v<Tin>) draws[base + q] = dist(gen);
                    else o[base + q] = (dist(gen) < 0.5f) ? R(-1.f) : R(1.f);
                }
            });
            if constexpr (is_cplx_v<Tin>) {
                std::complex<float> const kf = 2 * PI_F * std::complex<float>(0, 1);
                std::complex<R> const k(static_cast<R>(kf.real()), static_cast<R>(kf.imag()));
                int64_t const total = static_cast<int64_t>(draws.size()), chunk = 1 << 16;
                parallel_for((total + chunk - 1) / chunk, [&](int64_t c) {
                    for (int64_t q = c * chunk; q < std::min(total, (c + 1) * chunk); ++q) o[q] = std::exp(k * draws[q]);
                });
            }
        });
        e->progress_total = e->progress_fn ? num_random : 0;
        struct ProgressEnd {  // no reports outside this call, also after an exception
            kpm_engine* e;
            ~ProgressEnd() { e->progress_total = 0; }
        } progress_end{e};
        e->progress(-1);
        e->run_diag(Mmax, num_random, st.data(), false, nullptr, false);
        e->progress(num_random);
        e->progress_total = 0;
        e->reset_stats(Mmax, true, false, static_cast<double>(num_random) * e->nsys, 0);
        e->d_mu_avg.ensure(sizeof(double) * 2 * e->nsys * Mmax);
        KPM_CUDA(kpm::launch_average(e->d_mu.as<double>(), e->nsys, num_random, Mmax, e->d_mu_avg.as<double>(), e->stream));
        for (int s = 0; s < e->nsys; ++s) {
            double* m = e->d_mu_avg.as<double>() + 2 * s * Mmax;
            e->damp_device(m, Ms[s], 1, Mmax);
            e->spectral(m, Ms[s], 1, energy, ne, e->scale(s), out + s * ne);
        }
        e->finish_stats();
        e->calc_time = now_s() - t0;
    });
}

int kpm_calc_ldos(kpm_engine* e, const int64_t* idx, int64_t nidx, const double* energy, int64_t ne,
                  double broadening, double* out) {
    return guarded([&] {
        if (!e) fail(KPM_ERR_VALUE, "null engine");
        HostThreads host_threads(e->cfg.num_threads);
        if (e->nsys != 1) fail(KPM_ERR_VALUE, "LDOS needs a single-system engine");
        if (nidx < 1 || !idx) fail(KPM_ERR_VALUE, "no LDOS indices");
        double const t0 = now_s();
        std::vector<int32_t> ii;
        for (int64_t i = 0; i < nidx; ++i) {
            if (idx[i] < 0 || idx[i] >= e->rows) fail(KPM_ERR_RUNTIME, "LDOS index out of range");
            ii.push_back(static_cast<int32_t>(idx[i]));
        }
        auto const sc = e->scale(0);
        int64_t const M = required_moments(e->cfg.kernel, e->cfg.kernel_param, broadening / sc.a);
        e->optimize(ii, ii);
        std::vector<int32_t> pos = e->idx_src;
        bool const opt = e->cfg.optimal_size != 0 && e->reorders();
        e->run_diag(M, nidx, nullptr, false, &pos, opt);
        e->reset_stats(M, true, opt, static_cast<double>(nidx), 0);
        e->damp_device(e->d_mu.as<double>(), M, nidx, M);
        e->spectral(e->d_mu.as<double>(), M, static_cast<int>(nidx), energy, ne, sc, out);
        e->finish_stats();
        e->calc_time = now_s() - t0;
    });
}

int kpm_calc_ldos_batch(kpm_engine* e, const int64_t* sites, const double* energy, int64_t ne, double broadening,
                        double* out) {
    return guarded([&] {
        if (!e) fail(KPM_ERR_VALUE, "null engine");
        HostThreads host_threads(e->cfg.num_threads);
        if (!sites) fail(KPM_ERR_VALUE, "no LDOS sites");
        if (ne > 0 && (!energy || !out)) fail(KPM_ERR_VALUE, "null energy or output");
        for (int s = 0; s < e->nsys; ++s)
            if (sites[s] < 0 || sites[s] >= e->sys_rows(s)) fail(KPM_ERR_RUNTIME, "LDOS index out of range");
        double const t0 = now_s();
        e->compute_bounds();
        std::vector<int64_t> Ms(e->nsys);
        int64_t Mmax = 2;
        for (int s = 0; s < e->nsys; ++s) {
            Ms[s] = required_moments(e->cfg.kernel, e->cfg.kernel_param, broadening / e->scale(s).a);
            Mmax = std::max(Mmax, Ms[s]);
        }
        e->optimize({0}, {0});
        std::vector<int32_t> pos(e->nsys);
        for (int s = 0; s < e->nsys; ++s) pos[s] = e->map[e->sys_off[s] + sites[s]];
        e->run_diag(Mmax, 1, nullptr, false, &pos, false, true);
        e->reset_stats(Mmax, true, false, static_cast<double>(e->nsys), 0);
        for (int s = 0; s < e->nsys; ++s) {
            double* m = e->d_mu.as<double>() + 2 * s * Mmax;
            e->damp_device(m, Ms[s], 1, Mmax);
            e->spectral(m, Ms[s], 1, energy, ne, e->scale(s), out + s * ne);
        }
        e->finish_stats();
        e->calc_time = now_s() - t0;
    });
}

int kpm_calc_greens(kpm_engine* e, int64_t row, const int64_t* cols, int64_t ncols, const double* energy, int64_t ne,
                    double broadening, double* out) {
    return guarded([&] {
        if (!e) fail(KPM_ERR_VALUE, "null engine");
        HostThreads host_threads(e->cfg.num_threads);
        if (e->nsys != 1) fail(KPM_ERR_VALUE, "Green's function needs a single-system engine");
        if (ncols < 1 || !cols) fail(KPM_ERR_VALUE, "no Green's function columns");
        int64_t const size = e->rows;
        bool bad = row < 0 || row > size;
        for (int64_t j = 0; j < ncols; ++j) bad = bad || cols[j] < 0 || cols[j] > size;
        if (bad) fail(KPM_ERR_RUNTIME, "KPM::calc_greens(i,j): invalid value for i or j.");
        double const t0 = now_s();
        auto const sc = e->scale(0);
        int64_t const M = required_moments(e->cfg.kernel, e->cfg.kernel_param, broadening / sc.a);
        std::vector<int32_t> src{static_cast<int32_t>(row)}, dest;
        for (int64_t j = 0; j < ncols; ++j) dest.push_back(static_cast<int32_t>(cols[j]));
        e->optimize(src, dest);
        bool const opt = e->cfg.optimal_size != 0 && e->reorders();
        bool const diagonal = src == dest;
        e->d_energy.ensure(sizeof(double) * std::max<int64_t>(ne, 1));
        KPM_CUDA(cudaMemcpyAsync(e->d_energy.p, energy, sizeof(double) * ne, cudaMemcpyHostToDevice, e->stream));
        if (diagonal) {
            std::vector<int32_t> pos = e->idx_src;
            e->run_diag(M, 1, nullptr, false, &pos, opt);
            e->reset_stats(M, true, opt, 1.0, 0);
            e->damp_device(e->d_mu.as<double>(), M, 1, M);
            e->d_out.ensure(sizeof(double) * 2 * std::max<int64_t>(ne, 1));
            KPM_CUDA(kpm::launch_greens(e->d_mu.as<double>(), M, 1, e->d_energy.as<double>(), static_cast<int>(ne), sc.a,
                                        sc.b, e->d_out.as<double>(), e->stream));
            KPM_CUDA(cudaMemcpyAsync(out, e->d_out.p, sizeof(double) * 2 * ne, cudaMemcpyDeviceToHost, e->stream));
            KPM_CUDA(cudaStreamSynchronize(e->stream));
        } else {
            // MultiUnit off-diagonal recursion (calc_moments.hpp:102-114, collectors.cpp:60-76):
            // r0 = unit at src, collect r_n[dest_j] after every step
            int const vt = e->vtype;
            int const vb = kpm::vtype_bytes(vt);
            int64_t const nd = ncols;
            e->d_x0.ensure(static_cast<size_t>(e->rows) * vb);
            e->d_x1.ensure(static_cast<size_t>(e->rows) * vb);
            e->d_mu.ensure(sizeof(double) * 2 * nd * M);
            e->d_pos.ensure(sizeof(int32_t) * (nd + 1));
            KPM_CUDA(cudaMemcpyAsync(e->d_pos.p, e->idx_src.data(), sizeof(int32_t), cudaMemcpyHostToDevice, e->stream));
            int32_t* d_dest = e->d_pos.as<int32_t>() + 1;
            KPM_CUDA(cudaMemcpyAsync(d_dest, e->idx_dest.data(), sizeof(int32_t) * nd, cudaMemcpyHostToDevice, e->stream));
            KPM_CUDA(cudaMemsetAsync(e->d_x0.p, 0, static_cast<size_t>(e->rows) * vb, e->stream));
            KPM_CUDA(kpm::launch_set_units(vt, e->d_x0.p, e->d_pos.as<int32_t>(), 1, 1, e->rows, e->stream));
            kpm_engine::Shape sh{1, 1, 1, 1, 4096};
            int const ntiles = e->build_tiles(sh, true);
            std::vector<double> mu(static_cast<size_t>(2 * nd * M));
            // gather buffers: step n -> d_acc[n * nd]
            e->d_acc.ensure(sizeof(double) * 2 * nd * M);
            KPM_CUDA(cudaEventRecord(e->ev0, e->stream));
            KPM_CUDA(kpm::launch_gather_rows(vt, e->d_x0.p, d_dest, static_cast<int>(nd), e->d_acc.as<double>(), e->stream));
            kpm::OffStep a{};
            a.vtype = vt;
            a.E = 1;
            a.LPR = 1;
            a.col = e->d_col.as<int32_t>();
            a.val = e->d_val.p;
            a.W = e->W;
            a.batch_stride = e->rows;
            a.tiles = e->d_tiles.as<Tile>();
            a.num_tiles = ntiles;
            a.row_limit = static_cast<int32_t>(e->rows);
            a.gamma = nullptr;
            a.acc = nullptr;
            a.x = e->d_x0.p;
            a.y = e->d_x1.p;
            a.init = true;
            KPM_CUDA(kpm::launch_off_step(a, e->stream));
            KPM_CUDA(kpm::launch_gather_rows(vt, e->d_x1.p, d_dest, static_cast<int>(nd), e->d_acc.as<double>() + 2 * nd,
                                             e->stream));
            a.init = false;
            void* r0 = e->d_x0.p;
            void* r1 = e->d_x1.p;
            for (int64_t n = 2; n < M; ++n) {
                a.x = r1;
                a.y = r0;
                if (opt) {
                    int32_t const lim = e->optimal_size(n, M);
                    a.row_limit = lim;
                    a.num_tiles = static_cast<int>(std::min<int64_t>(ntiles, (lim + 4095) / 4096));
                }
                KPM_CUDA(kpm::launch_off_step(a, e->stream));
                std::swap(r0, r1);
                KPM_CUDA(kpm::launch_gather_rows(vt, r1, d_dest, static_cast<int>(nd), e->d_acc.as<double>() + 2 * nd * n,
                                                 e->stream));
            }
            KPM_CUDA(cudaEventRecord(e->ev1, e->stream));
            KPM_CUDA(cudaMemcpyAsync(mu.data(), e->d_acc.p, sizeof(double) * mu.size(), cudaMemcpyDeviceToHost, e->stream));
            KPM_CUDA(cudaStreamSynchronize(e->stream));
            float ms = 0;
            KPM_CUDA(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
            e->st.moments_time = ms * 1e-3;
            auto g = damping(e->cfg.kernel, e->cfg.kernel_param, M);
            std::vector<double> cm(static_cast<size_t>(2 * nd * M));  // [j][n]
            for (int64_t j = 0; j < nd; ++j)
                for (int64_t n = 0; n < M; ++n) {
                    double const h = n == 0 ? 0.5 : 1.0;
                    cm[2 * (j * M + n)] = mu[2 * (n * nd + j)] * h * g[n];
                    cm[2 * (j * M + n) + 1] = mu[2 * (n * nd + j) + 1] * h * g[n];
                }
            KPM_CUDA(cudaMemcpyAsync(e->d_mu.p, cm.data(), sizeof(double) * cm.size(), cudaMemcpyHostToDevice, e->stream));
            e->d_out.ensure(sizeof(double) * 2 * std::max<int64_t>(ne * nd, 1));
            KPM_CUDA(kpm::launch_greens(e->d_mu.as<double>(), M, static_cast<int>(nd), e->d_energy.as<double>(),
                                        static_cast<int>(ne), sc.a, sc.b, e->d_out.as<double>(), e->stream));
            KPM_CUDA(cudaMemcpyAsync(out, e->d_out.p, sizeof(double) * 2 * ne * nd, cudaMemcpyDeviceToHost, e->stream));
            KPM_CUDA(cudaStreamSynchronize(e->stream));
            e->reset_stats(M, false, opt, 1.0, 0);
        }
        e->finish_stats();
        e->calc_time = now_s() - t0;
    });
}

int kpm_moments(kpm_engine* e, int64_t num_moments, const double* alpha, int64_t alpha_size, const double* beta,
                int64_t beta_size, int64_t op_rows, const int32_t* op_indptr, const int32_t* op_indices,
                const double* op_values, double* out) {
    return guarded([&] {
        if (!e) fail(KPM_ERR_VALUE, "null engine");
        HostThreads host_threads(e->cfg.num_threads);
        if (e->nsys != 1) fail(KPM_ERR_VALUE, "moments() needs a single-system engine");
        int64_t const n = e->rows;
        // KPM.cpp:20-33 (checked in the reference's unordered_map order: operator, beta, alpha)
        if (op_rows != 0 && op_rows != n) fail(KPM_ERR_RUNTIME, "Size mismatch between the model Hamiltonian and the given argument 'operator'");
        if (beta_size != 0 && beta_size != n) fail(KPM_ERR_RUNTIME, "Size mismatch between the model Hamiltonian and the given argument 'beta'");
        if (alpha_size != n) fail(KPM_ERR_RUNTIME, "Size mismatch between the model Hamiltonian and the given argument 'alpha'");
        if (!scalar_complex(e->stype)) {  // KPM.cpp:35-48
            auto has_imag = [](double const* v, int64_t m) {
                for (int64_t i = 0; i < m; ++i) if (v[2 * i + 1] != 0) return true;
                return false;
            };
            if (op_rows && has_imag(op_values, op_indptr[op_rows])) fail(KPM_ERR_RUNTIME, "The model Hamiltonian is real, but the given argument 'operator' is complex");
            if (beta_size && has_imag(beta, beta_size)) fail(KPM_ERR_RUNTIME, "The model Hamiltonian is real, but the given argument 'beta' is complex");
            if (has_imag(alpha, alpha_size)) fail(KPM_ERR_RUNTIME, "The model Hamiltonian is real, but the given argument 'alpha' is complex");
        }
        double const t0 = now_s();
        int64_t const M = round_moments(num_moments);
        e->optimize({0}, {0});
        int const vt = e->vtype;
        int const vb = kpm::vtype_bytes(vt);
        // alpha in the Hamiltonian's scalar type (force_cast, collectors.cpp:38-49), original order
        std::vector<unsigned char> st(static_cast<size_t>(n) * scalar_bytes(e->stype));
        with_scalar(e->stype, [&](auto zi) {
            using Ts = decltype(zi);
            auto* o = reinterpret_cast<Ts*>(st.data());
            for (int64_t i = 0; i < n; ++i) o[i] = from_cd<Ts>(cd(alpha[2 * i], alpha[2 * i + 1]));
        });
        std::vector<double> mu(static_cast<size_t>(2 * M));
        if (beta_size == 0 && op_rows == 0) {
            e->run_diag(M, 1, st.data(), false, nullptr, false);
            KPM_CUDA(cudaMemcpyAsync(mu.data(), e->d_mu.p, sizeof(double) * 2 * M, cudaMemcpyDeviceToHost, e->stream));
            KPM_CUDA(cudaStreamSynchronize(e->stream));
            e->reset_stats(M, true, false, 1.0, 0);
        } else {
            // GenericCollector (collectors.cpp:38-58): mu_n = <beta| op r_n> = <gamma | r_n>, gamma = op^H beta
            std::vector<cd> bv(n), gv(n, cd(0, 0)), av(n);
            for (int64_t i = 0; i < n; ++i) {
                av[i] = cd(alpha[2 * i], alpha[2 * i + 1]);
                bv[i] = beta_size ? cd(beta[2 * i], beta[2 * i + 1]) : av[i];
            }
            if (op_rows) {
                for (int64_t r = 0; r < n; ++r)
                    for (int32_t k = op_indptr[r]; k < op_indptr[r + 1]; ++k) {
                        int32_t const c = op_indices[k];
                        if (c < 0 || c >= n) fail(KPM_ERR_VALUE, "operator column index out of range");
                        gv[c] += std::conj(cd(op_values[2 * k], op_values[2 * k + 1])) * bv[r];
                    }
            } else {
                gv = bv;
            }
            // mu0 = 0.5 <gamma|alpha> on the host (one dot), the rest fused in the step kernel
            cd mu0(0, 0);
            for (int64_t i = 0; i < n; ++i) mu0 += std::conj(gv[i]) * av[i];
            mu0 *= 0.5;
            std::vector<unsigned char> gam(static_cast<size_t>(n) * vb);
            with_vtype(vt, [&](auto zc) {
                using Tc = decltype(zc);
                auto* o = reinterpret_cast<Tc*>(gam.data());
                for (int64_t i = 0; i < n; ++i) o[e->map[i]] = from_cd<Tc>(gv[i]);
            });
            e->d_gamma.ensure(gam.size());
            KPM_CUDA(cudaMemcpyAsync(e->d_gamma.p, gam.data(), gam.size(), cudaMemcpyHostToDevice, e->stream));
            size_t const vbytes = static_cast<size_t>(n) * vb;
            e->d_x0.ensure(vbytes);
            e->d_x1.ensure(vbytes);
            void const* src = e->device_view(st.data(), st.size());
            KPM_CUDA(cudaMemsetAsync(e->d_x0.p, 0, vbytes, e->stream));
            KPM_CUDA(kpm::launch_scatter_starters(e->stype, vt, src, e->d_x0.p, e->d_map.as<int32_t>(),
                                                  e->d_sysoff.as<int64_t>(), 1, 1, 1, 1, n, e->stream));
            kpm_engine::Shape sh{1, 1, 1, 1, 4096};
            int const ntiles = e->build_tiles(sh, true);
            e->d_acc.ensure(sizeof(double) * 2 * M);
            KPM_CUDA(cudaMemsetAsync(e->d_acc.p, 0, sizeof(double) * 2 * M, e->stream));
            kpm::OffStep a{};
            a.vtype = vt;
            a.E = 1;
            a.LPR = 1;
            a.col = e->d_col.as<int32_t>();
            a.val = e->d_val.p;
            a.W = e->W;
            a.batch_stride = n;
            a.tiles = e->d_tiles.as<Tile>();
            a.num_tiles = ntiles;
            a.row_limit = static_cast<int32_t>(n);
            a.gamma = e->d_gamma.p;
            KPM_CUDA(cudaEventRecord(e->ev0, e->stream));
            a.x = e->d_x0.p;
            a.y = e->d_x1.p;
            a.init = true;
            a.acc = e->d_acc.as<double>() + 2;
            KPM_CUDA(kpm::launch_off_step(a, e->stream));
            a.init = false;
            void* r0 = e->d_x0.p;
            void* r1 = e->d_x1.p;
            for (int64_t k = 2; k < M; ++k) {
                a.x = r1;
                a.y = r0;
                a.acc = e->d_acc.as<double>() + 2 * k;
                KPM_CUDA(kpm::launch_off_step(a, e->stream));
                std::swap(r0, r1);
            }
            KPM_CUDA(cudaEventRecord(e->ev1, e->stream));
            KPM_CUDA(cudaMemcpyAsync(mu.data(), e->d_acc.p, sizeof(double) * 2 * M, cudaMemcpyDeviceToHost, e->stream));
            KPM_CUDA(cudaStreamSynchronize(e->stream));
            float ms = 0;
            KPM_CUDA(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
            e->st.moments_time = ms * 1e-3;
            mu[0] = mu0.real();
            mu[1] = mu0.imag();
            e->reset_stats(M, false, false, 1.0, 0);
        }
        auto g = damping(e->cfg.kernel, e->cfg.kernel_param, M);
        for (int64_t i = 0; i < num_moments; ++i) {
            out[2 * i] = mu[2 * i] * g[i];
            out[2 * i + 1] = mu[2 * i + 1] * g[i];
        }
        e->finish_stats();
        e->calc_time = now_s() - t0;
    });
}

namespace {

// The Kubo-Bastin moments matrix of system 0 (Core.cpp:119-145 up to normalize):
// mu[m][n] = sum_r L_m conj(R_n) / num_random with L_n = T_n(H~) V_l r and R_n = V_r T_n(H~) r
// (kpm/Moments.cpp:92-126), row and column 0 halved as the collectors store T_0 / 2,
// undamped; complex double, column n of M entries at mu + 2 n M. Returns the recursion and
// GEMM device times.
void conductivity_mu(kpm_engine* e, const float* left, const float* right, int64_t M, int64_t num_random,
                     int32_t gemm_mode, std::vector<double>& mu, double& rec_time, double& gemm_time) {
        if (e->nsys != 1) fail(KPM_ERR_VALUE, "conductivity needs a single-system engine");
        if (!left || !right) fail(KPM_ERR_VALUE, "null argument");
        if (num_random < 1) fail(KPM_ERR_VALUE, "num_random must be >= 1");
        if (M < 2) fail(KPM_ERR_VALUE, "num_moments must be >= 2");
        if (gemm_mode != 0 && gemm_mode != 1) fail(KPM_ERR_VALUE, "gemm_mode must be 0 (FP64) or 1 (tensor cores)");
        bool const tc = gemm_mode == 1;
        e->optimize({0}, {0});
        int64_t const n = e->rows;
        int const vt = e->vtype;
        int const vb = kpm::vtype_bytes(vt);
        int const W = e->W;
        // Velocity operators V = H o (x_i - x_j) in H's scalar type (kpm/Moments.cpp:132-155).
        // Left: applied to the random starter in the original order (Starter.cpp:66,78).
        // Right: applied to every collected vector, aligned with the reordered ELL of H~.
        std::vector<int32_t> const& hcol = e->h_col;  // host copy of the device ELL columns
        int const vs = kpm::vtype_vs(vt);
        std::vector<unsigned char> vr_ell(static_cast<size_t>(n) * W * vs * vb, 0);
        std::vector<unsigned char>& starters_l = e->h_starters;  // reused between calls (read in place)
        std::vector<unsigned char>& starters_r = e->h_starters_right;
        int64_t K = 1;
        // tensor-core GEMM: the collected vectors are kept as FP32 planes (re [, im])
        int const planes = kpm::vtype_complex(vt) ? 2 : 1;
        {   // vectors per batch: both sides keep M x n x K vectors
            size_t free_b = 0, total_b = 0;
            KPM_CUDA(cudaMemGetInfo(&free_b, &total_b));
            double const per_vec = 2.0 * static_cast<double>(M) * n * (tc ? 4 * planes : vb);
            int64_t kmax = static_cast<int64_t>(0.5 * static_cast<double>(free_b) / per_vec);
            if (kmax < 1) fail(KPM_ERR_RUNTIME, "not enough device memory for the conductivity moments");
            for (int64_t k : {16, 8, 4, 2, 1}) {
                kpm_engine::Shape sh = e->pick_shape(k);
                if (k <= kmax && k <= num_random && sh.K == k) { K = k; break; }
            }
        }
        kpm_engine::Shape sh = e->pick_shape(K);
        if (sh.K != K || sh.nbatch != 1) { K = 1; sh = kpm_engine::Shape{1, 1, 1, 1, 4096}; }
        int64_t const nrand_pad = ((num_random + K - 1) / K) * K;
        size_t const ssize = static_cast<size_t>(scalar_bytes(e->stype));
        starters_l.assign(static_cast<size_t>(nrand_pad) * n * ssize, 0);
        starters_r.assign(static_cast<size_t>(nrand_pad) * n * ssize, 0);
        with_scalar(e->stype, [&](auto zi) {
            using T = decltype(zi);
            using R = real_of<T>;
            auto const* hv = reinterpret_cast<T const*>(e->values.data());
            std::vector<T> vl(e->indices.size());
            // every entry writes its own slots: rows in parallel chunks
            std::atomic<bool> outside{false};
            int64_t const chunk = 1 << 14;
            parallel_for((n + chunk - 1) / chunk, [&](int64_t ch) {
                for (int64_t r = ch * chunk; r < std::min(n, (ch + 1) * chunk); ++r)
                    for (int32_t k = e->indptr[r]; k < e->indptr[r + 1]; ++k) {
                        int32_t const c = e->indices[k];
                        vl[k] = hv[k] * static_cast<T>(left[r] - left[c]);
                        cd const vrv = to_cd(hv[k]) * static_cast<double>(right[r] - right[c]);
                        int32_t const nr = e->map[r], nc = e->map[c];
                        int j = 0;
                        while (j < W && hcol[static_cast<size_t>(nr) * W + j] != nc) ++j;
                        if (j == W) {
                            outside = true;
                            continue;
                        }
                        with_vtype(vt, [&](auto zc) {
                            using Tc = decltype(zc);
                            Tc* o = reinterpret_cast<Tc*>(vr_ell.data()) + (static_cast<size_t>(nr) * W + j) * vs;
                            Tc const hi = from_cd<Tc>(vrv);
                            o[0] = hi;
                            if (vs == 2) o[1] = from_cd<Tc>(vrv - to_cd(hi));
                        });
                    }
            });
            if (outside) fail(KPM_ERR_RUNTIME, "internal: velocity entry outside the H~ pattern");
            // both starters own a default-seeded generator, so left and right draw the same r;
            // the draws stay in the reference's order (one sequence over vectors, then sites),
            // the rest (phases, the left velocity product) runs in parallel over vectors
            std::mt19937 gen;
            std::uniform_real_distribution<R> dist;
            std::vector<R> draws(static_cast<size_t>(num_random) * n);
            for (auto& d : draws) d = dist(gen);
            auto* sl = reinterpret_cast<T*>(starters_l.data());
            auto* sr = reinterpret_cast<T*>(starters_r.data());
            parallel_for(num_random, [&](int64_t v) {
                T* rv = sr + v * n;
                R const* dv = draws.data() + static_cast<size_t>(v) * n;
                for (int64_t i = 0; i < n; ++i) {
                    if constexpr (is_cplx_v<T>) {
                        std::complex<float> const kf = 2 * PI_F * std::complex<float>(0, 1);
                        std::complex<R> const kk(static_cast<R>(kf.real()), static_cast<R>(kf.imag()));
                        rv[i] = std::exp(kk * dv[i]);
                    } else {
                        rv[i] = (dv[i] < 0.5f) ? R(-1.f) : R(1.f);
                    }
                }
                for (int64_t r = 0; r < n; ++r) {
                    T acc = T(0);
                    for (int32_t k = e->indptr[r]; k < e->indptr[r + 1]; ++k) acc += vl[k] * rv[e->indices[k]];
                    sl[v * n + r] = acc;
                }
            });
        });
        // device buffers
        size_t const vec_bytes = static_cast<size_t>(n) * K * vb;
        DBuf d_v2, d_L, d_R, d_mu_acc, d_samples, d_sum, d_chem, d_res;
        d_v2.ensure(vr_ell.size());
        e->upload_host(d_v2.p, vr_ell.data(), vr_ell.size());
        // plane row stride: 16-byte multiple for the tensor maps
        int64_t const ld = ((n * K + 3) / 4) * 4;
        if (tc && (M > (int64_t{1} << 20) || n * K > (int64_t{1} << 31) - 64))
            fail(KPM_ERR_VALUE, "gemm_mode=1 needs num_moments <= 2^20 and rows x vectors < 2^31");
        size_t const plane_bytes = sizeof(float) * static_cast<size_t>(ld) * M;
        d_L.ensure(tc ? plane_bytes * planes : vec_bytes * M);
        d_R.ensure(tc ? plane_bytes * planes : vec_bytes * M);
        DBuf d_err;
        if (tc) {
            d_err.ensure(sizeof(int));
            KPM_CUDA(cudaMemsetAsync(d_err.p, 0, sizeof(int), e->stream));
        }
        e->d_x0.ensure(vec_bytes);
        e->d_x1.ensure(vec_bytes);
        d_mu_acc.ensure(sizeof(double) * 2 * M * M);
        KPM_CUDA(cudaMemsetAsync(d_mu_acc.p, 0, sizeof(double) * 2 * M * M, e->stream));
        int const ntiles = e->build_tiles(sh, true);
        rec_time = 0;
        auto recursion = [&](unsigned char const* host_starters, bool right_side) {
            void const* src = e->device_view(host_starters, static_cast<size_t>(K) * n * ssize);
            KPM_CUDA(cudaMemsetAsync(e->d_x0.p, 0, vec_bytes, e->stream));
            KPM_CUDA(kpm::launch_scatter_starters(e->stype, vt, src, e->d_x0.p, e->d_map.as<int32_t>(),
                                                  e->d_sysoff.as<int64_t>(), 1, K, static_cast<int>(K), 1, n, e->stream));
            kpm::DenseStep a{};
            a.vtype = vt;
            a.E = sh.E;
            a.LPR = sh.LPR;
            a.col = e->d_col.as<int32_t>();
            a.val = e->d_val.p;
            a.val2 = right_side ? d_v2.p : nullptr;
            a.W = W;
            a.tiles = e->d_tiles.as<Tile>();
            a.num_tiles = ntiles;
            unsigned char* store = static_cast<unsigned char*>(right_side ? d_R.p : d_L.p);
            KPM_CUDA(cudaEventRecord(e->ev0, e->stream));
            // init: r1 = H~ r0 / 2, store r0 (or V r0) as row 0; steps n = 2..M-1 store row n-1;
            // one extra step stores row M-1 (its recursion output is not used)
            void* r0 = e->d_x0.p;
            void* r1 = e->d_x1.p;
            for (int64_t step = 1; step <= M; ++step) {
                a.init = step == 1;
                a.x = step == 1 ? r0 : r1;
                a.y = step == 1 ? r1 : r0;
                if (tc) {
                    auto* re = reinterpret_cast<float*>(store) + ld * (step - 1);
                    a.zre = re;
                    a.zim = planes == 2 ? re + ld * M : nullptr;
                    a.zx = nullptr;
                    a.zv = nullptr;
                } else {
                    void* row = store + vec_bytes * (step - 1);
                    a.zx = right_side ? nullptr : row;
                    a.zv = right_side ? row : nullptr;
                }
                KPM_CUDA(kpm::launch_dense_step(a, e->stream));
                if (step > 1) std::swap(r0, r1);
            }
            KPM_CUDA(cudaEventRecord(e->ev1, e->stream));
            KPM_CUDA(cudaStreamSynchronize(e->stream));
            float ms = 0;
            KPM_CUDA(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
            rec_time += ms * 1e-3;
        };
        gemm_time = 0;
        for (int64_t b = 0; b < nrand_pad / K; ++b) {
            recursion(starters_l.data() + static_cast<size_t>(b) * K * n * ssize, false);
            recursion(starters_r.data() + static_cast<size_t>(b) * K * n * ssize, true);
            KPM_CUDA(cudaEventRecord(e->ev0, e->stream));
            // mu += L R^H: inner dimension = rows x K (rows n of both stores are [row][K])
            if (tc) {
                auto const* lre = d_L.as<float>();
                auto const* rre = d_R.as<float>();
                KPM_CUDA(kpm::launch_mu_gemm_tc(planes == 2, lre, planes == 2 ? lre + ld * M : nullptr, rre,
                                                planes == 2 ? rre + ld * M : nullptr, M, n * K, ld, 1,
                                                d_mu_acc.as<double>(), d_err.as<int>(), e->stream));
            } else {
                KPM_CUDA(kpm::launch_mu_gemm_fp64(vt, d_L.p, d_R.p, M, n * K, d_mu_acc.as<double>(), e->stream));
            }
            KPM_CUDA(cudaEventRecord(e->ev1, e->stream));
            KPM_CUDA(cudaStreamSynchronize(e->stream));
            float ms = 0;
            KPM_CUDA(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
            gemm_time += ms * 1e-3;
        }
        if (tc) {
            int herr = 0;
            KPM_CUDA(cudaMemcpy(&herr, d_err.p, sizeof(int), cudaMemcpyDeviceToHost));
            if (herr != 0) fail(KPM_ERR_TIMEOUT, "tensor-core moments GEMM: a bounded device wait expired");
        }
        // normalise by the vectors, halve row/column 0 (the collectors store T_0 / 2)
        mu.assign(static_cast<size_t>(2 * M * M), 0.0);
        KPM_CUDA(cudaMemcpy(mu.data(), d_mu_acc.p, sizeof(double) * mu.size(), cudaMemcpyDeviceToHost));
        for (int64_t c = 0; c < M; ++c)
            for (int64_t r = 0; r < M; ++r) {
                double f = 1.0 / static_cast<double>(num_random);
                if (r == 0) f *= 0.5;
                if (c == 0) f *= 0.5;
                mu[2 * (c * M + r)] *= f;
                mu[2 * (c * M + r) + 1] *= f;
            }
}

// KuboBastin (reconstruct.hpp:90-143) of a damped moments matrix over bounds.linspaced(num_points)
// of system 0, on the GPU in FP64; out: nmu complex values.
void kubo_bastin(kpm_engine* e, double const* mu, int64_t M, const double* chem, int64_t nmu, double temperature,
                 int64_t num_points, double* out) {
        if (num_points < 2) fail(KPM_ERR_VALUE, "num_points >= 2 required");
        if (nmu > 0 && (!chem || !out)) fail(KPM_ERR_VALUE, "null argument");
        auto const sc = e->scale(0);
        DBuf d_mu, d_samples, d_sum, d_chem, d_res;
        d_mu.ensure(sizeof(double) * 2 * M * M);
        KPM_CUDA(cudaMemcpyAsync(d_mu.p, mu, sizeof(double) * 2 * M * M, cudaMemcpyHostToDevice, e->stream));
        // energy samples: bounds.linspaced(num_points) scaled (reconstruct.hpp:101-103)
        auto const& bs = e->sys[0];
        std::vector<double> samples(num_points), chem_s(std::max<int64_t>(nmu, 1));
        for (int64_t i = 0; i < num_points; ++i)
            samples[i] = (bs.emin + (bs.emax - bs.emin) * static_cast<double>(i) / static_cast<double>(num_points - 1) - sc.b) / sc.a;
        samples[num_points - 1] = (bs.emax - sc.b) / sc.a;
        for (int64_t j = 0; j < nmu; ++j) chem_s[j] = (chem[j] - sc.b) / sc.a;
        double const smax = *std::max_element(samples.begin(), samples.end());
        double const smin = *std::min_element(samples.begin(), samples.end());
        double const coeff = (smax - smin) / static_cast<double>(2 * num_points);
        double const inv_kbt = sc.a / (static_cast<double>(8.6173303e-5f) * temperature);
        double const prefix = 4.0 / (sc.a * sc.a);
        d_samples.ensure(sizeof(double) * num_points);
        d_sum.ensure(sizeof(double) * 2 * num_points);
        d_chem.ensure(sizeof(double) * std::max<int64_t>(nmu, 1));
        d_res.ensure(sizeof(double) * 2 * std::max<int64_t>(nmu, 1));
        KPM_CUDA(cudaMemcpyAsync(d_samples.p, samples.data(), sizeof(double) * num_points, cudaMemcpyHostToDevice, e->stream));
        KPM_CUDA(cudaMemcpyAsync(d_chem.p, chem_s.data(), sizeof(double) * nmu, cudaMemcpyHostToDevice, e->stream));
        KPM_CUDA(kpm::launch_kubo_sum(d_mu.as<double>(), M, d_samples.as<double>(), static_cast<int>(num_points),
                                      d_sum.as<double>(), e->stream));
        KPM_CUDA(kpm::launch_kubo_integrate(d_sum.as<double>(), d_samples.as<double>(), static_cast<int>(num_points),
                                            d_chem.as<double>(), static_cast<int>(nmu), inv_kbt, coeff, prefix,
                                            d_res.as<double>(), e->stream));
        if (nmu > 0)
            KPM_CUDA(cudaMemcpyAsync(out, d_res.p, sizeof(double) * 2 * nmu, cudaMemcpyDeviceToHost, e->stream));
        KPM_CUDA(cudaStreamSynchronize(e->stream));
}

void apply_matrix_damping(kpm_engine* e, std::vector<double>& mu, int64_t M) {  // g_m g_n (Kernel.hpp:48-56)
    auto g = damping(e->cfg.kernel, e->cfg.kernel_param, M);
    for (int64_t c = 0; c < M; ++c)
        for (int64_t r = 0; r < M; ++r) {
            mu[2 * (c * M + r)] *= g[r] * g[c];
            mu[2 * (c * M + r) + 1] *= g[r] * g[c];
        }
}

}  // namespace

int kpm_calc_conductivity(kpm_engine* e, const float* left, const float* right, const double* chem, int64_t nmu,
                          double broadening, double temperature, int64_t num_random, int64_t num_points,
                          int32_t gemm_mode, double* out) {
    return guarded([&] {
        if (!e) fail(KPM_ERR_VALUE, "null engine");
        HostThreads host_threads(e->cfg.num_threads);
        if (!left || !right || (nmu > 0 && (!chem || !out))) fail(KPM_ERR_VALUE, "null argument");
        if (num_random < 1 || num_points < 2) fail(KPM_ERR_VALUE, "num_random >= 1 and num_points >= 2 required");
        double const t0 = now_s();
        auto const sc = e->scale(0);
        int64_t const M = required_moments(e->cfg.kernel, e->cfg.kernel_param, broadening / sc.a);
        std::vector<double> mu;
        double rec_time = 0, gemm_time = 0;
        conductivity_mu(e, left, right, M, num_random, gemm_mode, mu, rec_time, gemm_time);
        apply_matrix_damping(e, mu, M);
        kubo_bastin(e, mu.data(), M, chem, nmu, temperature, num_points, out);
        e->st.moments_time = rec_time + gemm_time;
        e->reset_stats(M, false, false, static_cast<double>(num_random) * 2, 0);
        e->finish_stats();
        e->st.gemm_time = gemm_time;
        e->calc_time = now_s() - t0;
    });
}

int kpm_conductivity_moments(kpm_engine* e, const float* left, const float* right, int64_t num_moments,
                             int64_t num_random, int32_t gemm_mode, double* out) {
    return guarded([&] {
        if (!e) fail(KPM_ERR_VALUE, "null engine");
        HostThreads host_threads(e->cfg.num_threads);
        if (!out) fail(KPM_ERR_VALUE, "null output");
        double const t0 = now_s();
        std::vector<double> mu;
        double rec_time = 0, gemm_time = 0;
        conductivity_mu(e, left, right, num_moments, num_random, gemm_mode, mu, rec_time, gemm_time);
        std::memcpy(out, mu.data(), sizeof(double) * mu.size());
        e->st.moments_time = rec_time + gemm_time;
        e->reset_stats(num_moments, false, false, static_cast<double>(num_random) * 2, 0);
        e->finish_stats();
        e->st.gemm_time = gemm_time;
        e->calc_time = now_s() - t0;
    });
}

int kpm_kubo_bastin(kpm_engine* e, const double* mu, int64_t num_moments, const double* chem, int64_t nmu,
                    double temperature, int64_t num_points, double* out) {
    return guarded([&] {
        if (!e || !mu) fail(KPM_ERR_VALUE, "null argument");
        if (e->nsys != 1) fail(KPM_ERR_VALUE, "conductivity needs a single-system engine");
        if (num_moments < 1) fail(KPM_ERR_VALUE, "num_moments must be >= 1");
        double const t0 = now_s();
        kubo_bastin(e, mu, num_moments, chem, nmu, temperature, num_points, out);
        e->calc_time = now_s() - t0;
    });
}

// Reverse-mode gradient of the averaged diagonal moments (no reference counterpart).
// Forward: v0 = r, v1 = S v0 / 2, v_k = S v_{k-1} - v_{k-2} (k <= N = M / 2), with
// mu_1 = <v1|v0>, mu_{2k} = 2<v_k|v_k> - mu_0, mu_{2k+1} = 2<v_{k+1}|v_k> - mu_1
// (calc_moments.hpp:35-58, collectors.cpp:6-36). For L = sum_n w_n mean_r mu_n the adjoint
// vectors lam_k = dL/dv_k obey the same recursion backwards,
//   lam_N = beta_N v_{N-1},  lam_k = S lam_{k+1} - lam_{k+2} + 2 alpha_k v_k + beta_k v_{k-1} + beta_{k+1} v_{k+1},
// alpha_k = 2 w_{2k} / R, beta_k = 2 w_{2k-1} / R, and
//   dL/dS = sum_{k=1}^{N-1} lam_{k+1} v_k^T + (lam_1 + c1 v0) v0^T / 2,  c1 = (w_1 - sum_k w_{2k-1}) / R,
// on the pattern of S (symmetric, so the kernel accumulates the transposed entry from the
// gather it already does). dL/dH = (2 / a) dL/dS with a, b frozen. Forward vectors are kept
// as checkpoint pairs (v_c, v_{c+1}) every `checkpoint` steps and recomputed per segment.
int kpm_adjoint_diag(kpm_engine* e, int64_t num_moments, int64_t num_vectors, const void* starters,
                     const double* dl_dmu, int64_t checkpoint, double* out_grad_values, double* out_grad_onsite,
                     int64_t* num_moments_out) {
    return guarded([&] {
        if (!e) fail(KPM_ERR_VALUE, "null engine");
        HostThreads host_threads(e->cfg.num_threads);
        if (!starters || !dl_dmu || !out_grad_values) fail(KPM_ERR_VALUE, "null argument");
        if (e->nsys != 1) fail(KPM_ERR_VALUE, "adjoint gradients need a single-system engine");
        if (kpm::vtype_complex(e->vtype) || e->stype == KPM_C64 || e->stype == KPM_C128)
            fail(KPM_ERR_VALUE, "adjoint gradients need a real Hamiltonian");
        if (num_vectors < 1) fail(KPM_ERR_VALUE, "num_vectors must be >= 1");
        if (checkpoint < 0) fail(KPM_ERR_VALUE, "checkpoint must be >= 0");
        double const t0 = now_s();
        int64_t const M = round_moments(num_moments);
        int64_t const N = M / 2;
        e->optimize({0}, {0});
        auto const sc = e->scale(0);
        int64_t const n = e->rows;
        int const vt = e->vtype;
        int const vb = kpm::vtype_bytes(vt);
        int const W = e->W;
        kpm_engine::Shape sh = e->pick_shape(num_vectors);
        int64_t const K = sh.K;
        size_t const vec = static_cast<size_t>(n) * K * vb;
        // segment length: at least 2 (a checkpoint pair is two consecutive vectors). Automatic:
        // the whole recursion when it fits in half the free memory (no checkpoint pass), else
        // sqrt(M / 2) (memory ~ 3 sqrt(M / 2) vectors, one extra forward pass)
        int64_t want = checkpoint;
        if (want == 0) {
            size_t free_b = 0, total_b = 0;
            KPM_CUDA(cudaMemGetInfo(&free_b, &total_b));
            want = static_cast<double>(N + 6) * vec <= 0.5 * static_cast<double>(free_b)
                       ? N
                       : static_cast<int64_t>(std::ceil(std::sqrt(static_cast<double>(N))));
        }
        int64_t const seg_len = std::max<int64_t>(2, std::min<int64_t>(want, N - 1));
        int64_t const nseg = N >= 2 ? (N - 2) / seg_len + 1 : 0;  // segments cover k = 1 .. N-1
        double const R = static_cast<double>(num_vectors);
        std::vector<double> alpha(N + 2, 0.0), beta(N + 2, 0.0);
        for (int64_t k = 1; k <= N - 1; ++k) alpha[k] = 2.0 * dl_dmu[2 * k] / R;
        for (int64_t k = 2; k <= N; ++k) beta[k] = 2.0 * dl_dmu[2 * k - 1] / R;
        double c1 = M > 1 ? dl_dmu[1] : 0.0;
        for (int64_t k = 2; k <= N; ++k) c1 -= dl_dmu[2 * k - 1];
        c1 /= R;

        sh.nbatch = 1;
        int const ntiles = e->build_tiles(sh, true);
        // checkpoint pairs, segment vectors v_{c+2} .. v_{c+seg_len+1}, two adjoint vectors,
        // two rolling forward vectors
        DBuf d_ck, d_seg, d_lam, d_roll, d_gt, d_gd;
        d_ck.ensure(vec * 2 * std::max<int64_t>(nseg, 1));
        d_seg.ensure(vec * seg_len);
        d_lam.ensure(vec * 2);
        d_roll.ensure(vec * 2);
        d_gt.ensure(sizeof(double) * n * W);  // gradient sums: FP64, or (hi, lo) FP32 pairs for FP32 vectors
        d_gd.ensure(sizeof(double) * n);
        KPM_CUDA(cudaMemsetAsync(d_gt.p, 0, d_gt.bytes, e->stream));
        KPM_CUDA(cudaMemsetAsync(d_gd.p, 0, d_gd.bytes, e->stream));
        auto* ck = static_cast<unsigned char*>(d_ck.p);
        auto* segb = static_cast<unsigned char*>(d_seg.p);
        auto* lamb = static_cast<unsigned char*>(d_lam.p);
        auto* roll = static_cast<unsigned char*>(d_roll.p);
        auto ckA = [&](int64_t j) { return ck + vec * (2 * j); };      // v_{j s}
        auto ckB = [&](int64_t j) { return ck + vec * (2 * j + 1); };  // v_{j s + 1}

        kpm::AdjStep base{};
        base.vtype = vt;
        base.E = sh.E;
        base.LPR = sh.LPR;
        base.col = e->d_col.as<int32_t>();
        base.val = e->d_val.p;
        base.W = W;
        base.tiles = e->d_tiles.as<Tile>();
        base.num_tiles = ntiles;
        auto step = [&](void const* x, void const* yprev, void* out, bool half) {  // out = S x - yprev
            kpm::AdjStep a = base;
            a.x = x;
            a.yprev = yprev;
            a.out = out;
            a.half = half;
            KPM_CUDA(kpm::launch_adj_step(a, e->stream));
        };

        size_t const ssize = static_cast<size_t>(scalar_bytes(e->stype));
        std::vector<unsigned char> stage(static_cast<size_t>(K) * n * ssize);
        KPM_CUDA(cudaEventRecord(e->ev0, e->stream));
        int64_t const nbatch = (num_vectors + K - 1) / K;
        for (int64_t b = 0; b < nbatch; ++b) {
            int64_t const v_first = b * K;
            int64_t const v_count = std::min<int64_t>(K, num_vectors - v_first);
            KPM_CUDA(cudaStreamSynchronize(e->stream));  // the previous batch's upload has been consumed
            std::fill(stage.begin(), stage.end(), 0);  // missing vectors of the last batch are zero
            std::memcpy(stage.data(), static_cast<unsigned char const*>(starters) + static_cast<size_t>(v_first) * n * ssize,
                        static_cast<size_t>(v_count) * n * ssize);
            void const* src = e->device_view(stage.data(), stage.size());
            KPM_CUDA(cudaMemsetAsync(ckA(0), 0, vec, e->stream));
            KPM_CUDA(kpm::launch_scatter_starters(e->stype, vt, src, ckA(0), e->d_map.as<int32_t>(),
                                                  e->d_sysoff.as<int64_t>(), 1, K, static_cast<int>(K), 1, n,
                                                  e->stream));
            // forward pass: checkpoints (v_c, v_{c+1}) for c = j * seg_len
            unsigned char* v0 = ckA(0);
            unsigned char* v1 = nseg > 0 ? ckB(0) : roll;
            step(v0, nullptr, v1, true);
            if (nseg > 1) {
                int64_t const last = (nseg - 1) * seg_len + 1;  // highest index needed
                auto fwd_ptr = [&](int64_t k) -> unsigned char* {
                    if (k % seg_len == 0 && k / seg_len < nseg) return ckA(k / seg_len);
                    if (k % seg_len == 1 && k / seg_len < nseg) return ckB(k / seg_len);
                    return roll + vec * (k % 2);
                };
                for (int64_t k = 1; k < last; ++k) step(fwd_ptr(k), fwd_ptr(k - 1), fwd_ptr(k + 1), false);
            }
            // backward pass, segment by segment from the end
            unsigned char* lam1 = nullptr;  // lam_{k+1}
            unsigned char* lam2 = nullptr;  // lam_{k+2} (nullptr = 0)
            for (int64_t j = nseg - 1; j >= 0; --j) {
                int64_t const c = j * seg_len;
                int64_t const kmax = std::min<int64_t>(c + seg_len, N - 1);
                auto sp = [&](int64_t k) -> unsigned char* {
                    if (k == c) return ckA(j);
                    if (k == c + 1) return ckB(j);
                    return segb + vec * (k - c - 2);
                };
                for (int64_t k = c + 1; k <= kmax; ++k) step(sp(k), sp(k - 1), sp(k + 1), false);
                if (lam1 == nullptr) {  // lam_N = beta_N v_{N-1}
                    lam1 = lamb;
                    KPM_CUDA(kpm::launch_axpby(vt, n * K, beta[N], sp(N - 1), 0.0, nullptr, lam1, e->stream));
                }
                for (int64_t k = kmax; k > c; --k) {
                    unsigned char* out = lam2 != nullptr ? lam2 : (lam1 == lamb ? lamb + vec : lamb);
                    kpm::AdjStep a = base;
                    a.x = lam1;
                    a.yprev = lam2;
                    a.out = out;
                    a.half = false;
                    a.v0 = sp(k);
                    a.a0 = 2.0 * alpha[k];
                    a.vm = sp(k - 1);
                    a.am = beta[k];
                    a.vp = sp(k + 1);
                    a.ap = beta[k + 1];
                    a.g = sp(k);
                    a.gt = d_gt.p;
                    a.gd = d_gd.p;
                    KPM_CUDA(kpm::launch_adj_step(a, e->stream));
                    lam2 = lam1;
                    lam1 = out;
                }
            }
            // (lam_1 + c1 v0) v0^T / 2
            unsigned char* u = (lam1 == lamb) ? lamb + vec : lamb;
            if (lam1 != nullptr)
                KPM_CUDA(kpm::launch_axpby(vt, n * K, 0.5, lam1, 0.5 * c1, v0, u, e->stream));
            else
                KPM_CUDA(kpm::launch_axpby(vt, n * K, 0.5 * c1, v0, 0.0, nullptr, u, e->stream));
            kpm::AdjStep a = base;
            a.x = u;
            a.g = v0;
            a.gt = d_gt.p;
            a.gd = d_gd.p;
            KPM_CUDA(kpm::launch_adj_step(a, e->stream));
        }
        KPM_CUDA(cudaEventRecord(e->ev1, e->stream));
        std::vector<unsigned char> gt_raw(d_gt.bytes), gd_raw(d_gd.bytes);
        std::vector<int32_t> hcol(static_cast<size_t>(n) * W);
        KPM_CUDA(cudaMemcpyAsync(gt_raw.data(), d_gt.p, gt_raw.size(), cudaMemcpyDeviceToHost, e->stream));
        KPM_CUDA(cudaMemcpyAsync(gd_raw.data(), d_gd.p, gd_raw.size(), cudaMemcpyDeviceToHost, e->stream));
        KPM_CUDA(cudaMemcpyAsync(hcol.data(), e->d_col.p, sizeof(int32_t) * hcol.size(), cudaMemcpyDeviceToHost, e->stream));
        KPM_CUDA(cudaStreamSynchronize(e->stream));
        float ms = 0;
        KPM_CUDA(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
        std::vector<double> gt(static_cast<size_t>(n) * W), gd(static_cast<size_t>(n));
        if (vt == kpm::V_F32) {  // (hi, lo) FP32 pairs
            std::vector<float> pt(2 * gt.size()), pd(2 * gd.size());
            std::memcpy(pt.data(), gt_raw.data(), sizeof(float) * pt.size());
            std::memcpy(pd.data(), gd_raw.data(), sizeof(float) * pd.size());
            for (size_t i = 0; i < gt.size(); ++i) gt[i] = static_cast<double>(pt[2 * i]) + pt[2 * i + 1];
            for (size_t i = 0; i < gd.size(); ++i) gd[i] = static_cast<double>(pd[2 * i]) + pd[2 * i + 1];
        } else {
            std::memcpy(gt.data(), gt_raw.data(), sizeof(double) * gt.size());
            std::memcpy(gd.data(), gd_raw.data(), sizeof(double) * gd.size());
        }
        // gt[p][t] holds G[col(p, t)][p]: entry (i, j) of the input is found in row map[j]
        double const f = 2.0 / sc.a;
        for (int64_t i = 0; i < n; ++i)
            for (int32_t k = e->indptr[i]; k < e->indptr[i + 1]; ++k) {
                int32_t const ni = e->map[i], nj = e->map[e->indices[k]];
                int t = 0;
                while (t < W && hcol[static_cast<size_t>(nj) * W + t] != ni) ++t;
                if (t == W) fail(KPM_ERR_RUNTIME, "internal: adjoint entry outside the S pattern");
                out_grad_values[k] = f * (ni == nj ? gd[ni] : gt[static_cast<size_t>(nj) * W + t]);
            }
        if (out_grad_onsite)
            for (int64_t i = 0; i < n; ++i) out_grad_onsite[i] = f * gd[e->map[i]];
        e->reset_stats(M, true, false, static_cast<double>(num_vectors), 0);
        e->st.moments_time = ms * 1e-3;
        e->finish_stats();
        e->calc_time = now_s() - t0;
        if (num_moments_out) *num_moments_out = M;
    });
}

// Reverse-mode gradient of a loss of the Kubo-Bastin moments matrix (real Hamiltonians, FP64
// recursion). With t^l_m = T_m(H~) V_l r, t^r_n = T_n(H~) r and u_n = V_r t^r_n (row and column
// 0 halved as the collectors store them, kpm/default/collectors.cpp:82-107),
//   mu_mn = (1/R) sum_r h_m h_n <t^l_m, u_n>,   L = sum_mn dl_dmu[m][n] mu_mn,
// the cotangents of the stored vectors are A_m = sum_n C_mn u_n and B_n = sum_m C_mn t^l_m with
// C_mn = dl_dmu[m][n] h_m h_n / R (two FP64 combinations on the GPU). Each side then runs the
// adjoint of its Chebyshev chain (t_0 = s, t_1 = S s / 2, t_{m+1} = S t_m - t_{m-1}, S = 2 H~):
//   lam_m = a_m + S lam_{m+1} - lam_{m+2},  lam_0 = a_0 + S lam_1 / 2 - lam_2,
//   dL/dS += sum_{m>=1} lam_{m+1} t_m^T + lam_1 t_0^T / 2,
// with sources a_m = A_m on the left and a_n = V_r^T B_n = -V_r B_n on the right (V is
// antisymmetric for a real H). The velocity operators V = H o (x_i - x_j) depend on H too:
// dL/dV_l = lam^l_0 r^T and dL/dV_r = sum_n B_n (t^r_n)^T on the pattern of H. Everything stays on
// the device (every vector of both chains is kept: 5 M x rows x K doubles).
int kpm_adjoint_conductivity(kpm_engine* e, const float* left, const float* right, int64_t num_moments,
                             int64_t num_vectors, const void* starters, const double* dl_dmu, double* out_mu,
                             double* out_grad_values, double* out_grad_onsite) {
    return guarded([&] {
        if (!e) fail(KPM_ERR_VALUE, "null engine");
        HostThreads host_threads(e->cfg.num_threads);
        if (!left || !right || !starters) fail(KPM_ERR_VALUE, "null argument");
        if ((dl_dmu == nullptr) != (out_grad_values == nullptr))
            fail(KPM_ERR_VALUE, "dl_dmu and out_grad_values go together");
        if (e->nsys != 1) fail(KPM_ERR_VALUE, "conductivity gradients need a single-system engine");
        if (e->stype == KPM_C64 || e->stype == KPM_C128 || e->vtype != kpm::V_F64)
            fail(KPM_ERR_VALUE, "conductivity gradients need a real Hamiltonian and the FP64 recursion "
                                "(float64 H, or precision fp64)");
        if (num_vectors < 1) fail(KPM_ERR_VALUE, "num_vectors must be >= 1");
        int64_t const M = num_moments;
        if (M < 3) fail(KPM_ERR_VALUE, "num_moments must be >= 3");
        double const t0 = now_s();
        e->optimize({0}, {0});
        auto const sc = e->scale(0);
        int64_t const n = e->rows;
        int const vt = kpm::V_F64;
        int const W = e->W;
        kpm_engine::Shape sh = e->pick_shape(num_vectors);
        int64_t const K = sh.K;
        int64_t const I = n * K;
        size_t const vec = sizeof(double) * static_cast<size_t>(I);
        {
            size_t free_b = 0, total_b = 0;
            KPM_CUDA(cudaMemGetInfo(&free_b, &total_b));
            if (static_cast<double>(5 * M + 8) * vec > 0.8 * static_cast<double>(free_b))
                fail(KPM_ERR_RUNTIME, "not enough device memory to keep both Chebyshev chains (5 x num_moments x rows "
                                      "x vectors doubles)");
        }
        // velocity operators V = H o (x_i - x_j) on the reordered ELL pattern of S (kpm/Moments.cpp:132-155;
        // float coordinate differences, KPM.cpp:140-145)
        std::vector<int32_t> const& hcol = e->h_col;
        std::vector<double> vl_ell(static_cast<size_t>(n) * W, 0.0), vr_ell(static_cast<size_t>(n) * W, 0.0);
        with_scalar(e->stype, [&](auto zi) {
            using T = decltype(zi);
            auto const* hv = reinterpret_cast<T const*>(e->values.data());
            for (int64_t r = 0; r < n; ++r)
                for (int32_t k = e->indptr[r]; k < e->indptr[r + 1]; ++k) {
                    int32_t const c = e->indices[k];
                    int32_t const nr = e->map[r], nc = e->map[c];
                    int j = 0;
                    while (j < W && hcol[static_cast<size_t>(nr) * W + j] != nc) ++j;
                    if (j == W) fail(KPM_ERR_RUNTIME, "internal: entry outside the S pattern");
                    size_t const q = static_cast<size_t>(nr) * W + j;
                    double const h = to_cd(hv[k]).real();
                    vl_ell[q] = h * static_cast<double>(left[r] - left[c]);
                    vr_ell[q] = h * static_cast<double>(right[r] - right[c]);
                }
        });
        DBuf d_vl, d_vr, d_tl, d_tr, d_u, d_a, d_b, d_lam, d_tmp, d_r0, d_gs, d_gsd, d_gvl, d_gvr, d_gvd, d_c, d_mu;
        d_vl.ensure(sizeof(double) * vl_ell.size());
        d_vr.ensure(sizeof(double) * vr_ell.size());
        e->upload_host(d_vl.p, vl_ell.data(), sizeof(double) * vl_ell.size());
        e->upload_host(d_vr.p, vr_ell.data(), sizeof(double) * vr_ell.size());
        d_tl.ensure(vec * M);
        d_tr.ensure(vec * M);
        d_u.ensure(vec * M);
        bool const grad = dl_dmu != nullptr;
        if (grad) {
            d_a.ensure(vec * M);
            d_b.ensure(vec * M);
        }
        d_lam.ensure(vec * 3);
        d_tmp.ensure(vec);
        d_r0.ensure(vec);
        size_t const gs_bytes = sizeof(double) * static_cast<size_t>(n) * W;
        for (DBuf* b : {&d_gs, &d_gvl, &d_gvr}) {
            b->ensure(gs_bytes);
            KPM_CUDA(cudaMemsetAsync(b->p, 0, gs_bytes, e->stream));
        }
        d_gsd.ensure(sizeof(double) * n);
        d_gvd.ensure(sizeof(double) * n);  // diagonal of the velocity gradients: unused (V_ii = 0)
        KPM_CUDA(cudaMemsetAsync(d_gsd.p, 0, sizeof(double) * n, e->stream));
        KPM_CUDA(cudaMemsetAsync(d_gvd.p, 0, sizeof(double) * n, e->stream));
        d_mu.ensure(sizeof(double) * 2 * M * M);
        KPM_CUDA(cudaMemsetAsync(d_mu.p, 0, sizeof(double) * 2 * M * M, e->stream));
        // C_mn = dl_dmu[m][n] h_m h_n / R, and its transpose
        double const R = static_cast<double>(num_vectors);
        std::vector<double> c, ct;
        if (grad) {
            c.resize(static_cast<size_t>(M) * M);
            ct.resize(static_cast<size_t>(M) * M);
            for (int64_t m = 0; m < M; ++m)
                for (int64_t q = 0; q < M; ++q) {
                    double const v = dl_dmu[m * M + q] * (m == 0 ? 0.5 : 1.0) * (q == 0 ? 0.5 : 1.0) / R;
                    c[m * M + q] = v;
                    ct[q * M + m] = v;
                }
            d_c.ensure(sizeof(double) * 2 * M * M);
            KPM_CUDA(cudaMemcpyAsync(d_c.p, c.data(), sizeof(double) * M * M, cudaMemcpyHostToDevice, e->stream));
            KPM_CUDA(cudaMemcpyAsync(d_c.as<double>() + M * M, ct.data(), sizeof(double) * M * M,
                                     cudaMemcpyHostToDevice, e->stream));
        }
        sh.nbatch = 1;
        int const ntiles = e->build_tiles(sh, true);
        kpm::AdjStep base{};
        base.vtype = vt;
        base.E = sh.E;
        base.LPR = sh.LPR;
        base.col = e->d_col.as<int32_t>();
        base.val = e->d_val.p;
        base.W = W;
        base.tiles = e->d_tiles.as<Tile>();
        base.num_tiles = ntiles;
        auto* tl = static_cast<unsigned char*>(d_tl.p);
        auto* tr = static_cast<unsigned char*>(d_tr.p);
        auto* u = static_cast<unsigned char*>(d_u.p);
        auto vrow = [&](unsigned char* b, int64_t m) { return b + vec * m; };
        auto apply_v = [&](void const* vals, void const* x, void* out) {  // out = V x on the pattern of S
            kpm::AdjStep a = base;
            a.val = vals;
            a.x = x;
            a.out = out;
            KPM_CUDA(kpm::launch_adj_step(a, e->stream));
        };
        auto chain = [&](unsigned char* t, void const* start) {  // t_0 .. t_{M-1}
            KPM_CUDA(cudaMemcpyAsync(t, start, vec, cudaMemcpyDeviceToDevice, e->stream));
            kpm::AdjStep a = base;
            a.x = t;
            a.out = vrow(t, 1);
            a.half = true;
            KPM_CUDA(kpm::launch_adj_step(a, e->stream));
            for (int64_t m = 1; m + 1 < M; ++m) {
                a.x = vrow(t, m);
                a.yprev = vrow(t, m - 1);
                a.out = vrow(t, m + 1);
                a.half = false;
                KPM_CUDA(kpm::launch_adj_step(a, e->stream));
            }
        };
        // the adjoint of a chain with sources a_m (rows of `src` times src_scale), S gradient into
        // d_gs / d_gsd; returns the buffer holding lam_0
        unsigned char* lamb = static_cast<unsigned char*>(d_lam.p);
        auto adjoint = [&](unsigned char* t, unsigned char* src, double src_scale) -> unsigned char* {
            unsigned char* l1 = nullptr;  // lam_{m+1}
            unsigned char* l2 = nullptr;  // lam_{m+2}
            auto fresh = [&]() {
                for (int q = 0; q < 3; ++q) {
                    unsigned char* b = lamb + vec * q;
                    if (b != l1 && b != l2) return b;
                }
                return lamb;
            };
            for (int64_t m = M - 1; m >= 0; --m) {
                unsigned char* out = fresh();
                if (l1 != nullptr) {
                    kpm::AdjStep a = base;
                    a.v0 = vrow(src, m);
                    a.a0 = src_scale;
                    a.x = l1;
                    a.yprev = l2;
                    a.half = (m == 0);
                    // dL/dS += lam_{m+1} t_m^T (m >= 1); lam_1 t_0^T / 2 at m = 0 (g = t_0 / 2)
                    if (m >= 1) {
                        a.g = vrow(t, m);
                    } else {
                        KPM_CUDA(kpm::launch_axpby(vt, I, 0.5, vrow(t, 0), 0.0, nullptr, d_tmp.p, e->stream));
                        a.g = d_tmp.p;
                    }
                    a.gt = d_gs.p;
                    a.gd = d_gsd.p;
                    a.out = out;
                    KPM_CUDA(kpm::launch_adj_step(a, e->stream));
                } else {  // lam_{M-1} = a_{M-1}
                    KPM_CUDA(kpm::launch_axpby(vt, I, src_scale, vrow(src, m), 0.0, nullptr, out, e->stream));
                }
                l2 = l1;
                l1 = out;
            }
            return l1;
        };
        auto grad_v = [&](void const* x, void const* g, void* gt) {  // gt[p][j] += x[col_j] . g[p]
            kpm::AdjStep a = base;
            a.x = x;
            a.g = g;
            a.gt = gt;
            a.gd = d_gvd.p;
            KPM_CUDA(kpm::launch_adj_step(a, e->stream));
        };

        size_t const ssize = static_cast<size_t>(scalar_bytes(e->stype));
        std::vector<unsigned char> stage(static_cast<size_t>(K) * n * ssize);
        int64_t const nbatch = (num_vectors + K - 1) / K;
        KPM_CUDA(cudaEventRecord(e->ev0, e->stream));
        for (int64_t bt = 0; bt < nbatch; ++bt) {
            int64_t const v_first = bt * K;
            int64_t const v_count = std::min<int64_t>(K, num_vectors - v_first);
            KPM_CUDA(cudaStreamSynchronize(e->stream));  // the previous batch's upload has been consumed
            std::fill(stage.begin(), stage.end(), 0);
            std::memcpy(stage.data(), static_cast<unsigned char const*>(starters) + static_cast<size_t>(v_first) * n * ssize,
                        static_cast<size_t>(v_count) * n * ssize);
            void const* src = e->device_view(stage.data(), stage.size());
            KPM_CUDA(cudaMemsetAsync(d_r0.p, 0, vec, e->stream));
            KPM_CUDA(kpm::launch_scatter_starters(e->stype, vt, src, d_r0.p, e->d_map.as<int32_t>(),
                                                  e->d_sysoff.as<int64_t>(), 1, K, static_cast<int>(K), 1, n, e->stream));
            // forward: t^l from V_l r, t^r from r, u_n = V_r t^r_n
            apply_v(d_vl.p, d_r0.p, d_tmp.p);
            chain(tl, d_tmp.p);
            chain(tr, d_r0.p);
            for (int64_t m = 0; m < M; ++m) apply_v(d_vr.p, vrow(tr, m), vrow(u, m));
            // mu_mn += sum <t^l_m, u_n> (the halved row / column 0 and 1/R are applied on the host)
            KPM_CUDA(kpm::launch_mu_gemm_fp64(vt, tl, u, M, I, d_mu.as<double>(), e->stream));
            if (!grad) continue;
            auto* A = static_cast<unsigned char*>(d_a.p);
            auto* B = static_cast<unsigned char*>(d_b.p);
            // A_m = sum_n C_mn u_n ; B_n = sum_m C_mn t^l_m
            KPM_CUDA(kpm::launch_dense_combine(d_c.as<double>(), reinterpret_cast<double const*>(u),
                                               reinterpret_cast<double*>(A), static_cast<int>(M), I, e->stream));
            KPM_CUDA(kpm::launch_dense_combine(d_c.as<double>() + M * M, reinterpret_cast<double const*>(tl),
                                               reinterpret_cast<double*>(B), static_cast<int>(M), I, e->stream));
            // left adjoint first: A is then free to hold the right side's sources V_r B_n
            unsigned char* lam0 = adjoint(tl, A, 1.0);
            grad_v(lam0, d_r0.p, d_gvl.p);  // dL/dV_l = lam^l_0 r^T
            for (int64_t q = 0; q < M; ++q) {
                grad_v(vrow(B, q), vrow(tr, q), d_gvr.p);  // dL/dV_r += B_q (t^r_q)^T
                apply_v(d_vr.p, vrow(B, q), vrow(A, q));   // A_q <- V_r B_q (sources, scaled by -1)
            }
            adjoint(tr, A, -1.0);
        }
        KPM_CUDA(cudaEventRecord(e->ev1, e->stream));
        std::vector<double> mu(static_cast<size_t>(2) * M * M);
        KPM_CUDA(cudaMemcpyAsync(mu.data(), d_mu.p, sizeof(double) * mu.size(), cudaMemcpyDeviceToHost, e->stream));
        std::vector<double> gs(static_cast<size_t>(n) * W), gsd(n), gvl(static_cast<size_t>(n) * W),
            gvr(static_cast<size_t>(n) * W);
        if (grad) {
            KPM_CUDA(cudaMemcpyAsync(gs.data(), d_gs.p, gs_bytes, cudaMemcpyDeviceToHost, e->stream));
            KPM_CUDA(cudaMemcpyAsync(gsd.data(), d_gsd.p, sizeof(double) * n, cudaMemcpyDeviceToHost, e->stream));
            KPM_CUDA(cudaMemcpyAsync(gvl.data(), d_gvl.p, gs_bytes, cudaMemcpyDeviceToHost, e->stream));
            KPM_CUDA(cudaMemcpyAsync(gvr.data(), d_gvr.p, gs_bytes, cudaMemcpyDeviceToHost, e->stream));
        }
        KPM_CUDA(cudaStreamSynchronize(e->stream));
        float ms = 0;
        KPM_CUDA(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
        if (out_mu)  // mu[m][n] (real part: zero imaginary part for a real H and real starters)
            for (int64_t m = 0; m < M; ++m)
                for (int64_t q = 0; q < M; ++q)
                    out_mu[m * M + q] = mu[2 * (q * M + m)] * (m == 0 ? 0.5 : 1.0) * (q == 0 ? 0.5 : 1.0) / R;
        if (grad) {
            // gt[p][t] holds the gradient of the transposed entry (col(p, t), p): the stored entry
            // (i, j) is found at slot (map[j], t) with col = map[i]
            double const f = 2.0 / sc.a;
            for (int64_t r = 0; r < n; ++r)
                for (int32_t k = e->indptr[r]; k < e->indptr[r + 1]; ++k) {
                    int32_t const c = e->indices[k];
                    int32_t const ni = e->map[r], nj = e->map[c];
                    if (c == r) {
                        out_grad_values[k] = f * gsd[ni];
                        continue;
                    }
                    int t = 0;
                    while (t < W && hcol[static_cast<size_t>(nj) * W + t] != ni) ++t;
                    if (t == W) fail(KPM_ERR_RUNTIME, "internal: adjoint entry outside the S pattern");
                    size_t const q = static_cast<size_t>(nj) * W + t;
                    // V = H o (x_i - x_j): dL/dH_ij += (x_i - x_j) dL/dV_ij on either side
                    double const dl = static_cast<double>(left[r] - left[c]);
                    double const dr = static_cast<double>(right[r] - right[c]);
                    out_grad_values[k] = f * gs[q] + dl * gvl[q] + dr * gvr[q];
                }
            if (out_grad_onsite)
                for (int64_t i = 0; i < n; ++i) out_grad_onsite[i] = f * gsd[e->map[i]];
        }
        e->reset_stats(M, false, false, static_cast<double>(num_vectors), 0);
        e->st.moments_time = ms * 1e-3;
        e->finish_stats();
        e->calc_time = now_s() - t0;
    });
}

int kpm_get_stats(kpm_engine* e, kpm_stats* out) {
    return guarded([&] {
        if (!e || !out) fail(KPM_ERR_VALUE, "null argument");
        *out = e->st;
        out->call_time = e->calc_time;
    });
}

int kpm_report(kpm_engine* e, int32_t shortform, char* buf, int64_t size) {
    return guarded([&] {
        if (!e || !buf || size < 1) fail(KPM_ERR_VALUE, "null argument");
        auto const& s = e->st;
        char line[512];
        std::string r;
        auto const& b = e->sys.empty() ? kpm_engine::Sys{} : e->sys[0];
        // Bounds::report (Bounds.cpp:33-39) + Stats::report (Stats.cpp:9-28, 67-69)
        if (shortform) {
            std::snprintf(line, sizeof line, "%.2f, %.2f, %d [%s] ", b.emin, b.emax, b.loops, pretty_time(s.bounds_time).c_str());
            r += line;
            double const removed = s.nnz ? 100.0 * static_cast<double>(s.nnz - s.opt_nnz) / static_cast<double>(s.nnz) : 0.0;
            std::snprintf(line, sizeof line, "%.0f%%%s [%s] ", removed, s.uses_full_system ? "" : "*", pretty_time(s.hamiltonian_time).c_str());
            r += line;
            std::snprintf(line, sizeof line, "%s @ %seps [%s] ", with_suffix(static_cast<double>(s.num_moments)).c_str(),
                          with_suffix(s.eps).c_str(), pretty_time(s.moments_time).c_str());
            r += line;
            r += "|";
        } else {
            std::snprintf(line, sizeof line, "Spectrum bounds found (%.2f, %.2f eV) using Lanczos procedure with %d loops", b.emin, b.emax, b.loops);
            char l2[640];
            std::snprintf(l2, sizeof l2, "- %-80s | %s\n", line, pretty_time(s.bounds_time).c_str());
            r += l2;
            double const removed = s.nnz ? 100.0 * static_cast<double>(s.nnz - s.opt_nnz) / static_cast<double>(s.nnz) : 0.0;
            std::snprintf(line, sizeof line, "The reordering optimization was able to remove %.0f%%%s of the workload", removed, s.uses_full_system ? "" : "*");
            std::snprintf(l2, sizeof l2, "- %-80s | %s\n", line, pretty_time(s.hamiltonian_time).c_str());
            r += l2;
            std::snprintf(line, sizeof line, "KPM calculated %s moments at %s non-zero elements per second",
                          with_suffix(static_cast<double>(s.num_moments)).c_str(), with_suffix(s.eps).c_str());
            std::snprintf(l2, sizeof l2, "- %-80s | %s\n", line, pretty_time(s.moments_time).c_str());
            r += l2;
            r += "Total time:";
        }
        r += " " + pretty_time(e->calc_time);
        std::strncpy(buf, r.c_str(), static_cast<size_t>(size - 1));
        buf[size - 1] = 0;
    });
}

int kpm_optimized_hamiltonian(kpm_engine* e, const int32_t* src, int64_t n_src, const int32_t* dest, int64_t n_dest,
                              int32_t reorder, int32_t* oip, int32_t* oix, void* ov, int64_t* onnz, int32_t* omap,
                              int32_t* oslices, int64_t* onslices, int32_t* osrc, int32_t* odest, int64_t* offsets) {
    return guarded([&] {
        if (!e) fail(KPM_ERR_VALUE, "null engine");
        HostThreads host_threads(e->cfg.num_threads);
        if (e->nsys != 1) fail(KPM_ERR_VALUE, "needs a single-system engine");
        if (n_src < 1 || n_dest < 1) fail(KPM_ERR_VALUE, "empty index lists");
        for (int64_t i = 0; i < n_src; ++i) if (src[i] < 0 || src[i] >= e->rows) fail(KPM_ERR_VALUE, "src index out of range");
        for (int64_t i = 0; i < n_dest; ++i) if (dest[i] < 0 || dest[i] >= e->rows) fail(KPM_ERR_VALUE, "dest index out of range");
        auto const sc = e->scale(0);
        std::vector<int32_t> s(src, src + n_src), d(dest, dest + n_dest);
        std::vector<int32_t> ip{0}, ix, borders;
        std::vector<int32_t> saved_map = e->map;
        e->map.assign(e->rows, 0);
        // in H's own scalar type: the reference's arithmetic, bit for bit
        with_scalar(e->stype, [&](auto z) {
            using T = decltype(z);
            std::vector<T> vals;
            e->reorder_system<T, T>(0, s, sc, reorder != 0, ip, ix, vals, &borders);
            std::memcpy(ov, vals.data(), vals.size() * sizeof(T));
        });
        std::copy(ip.begin(), ip.end(), oip);
        std::copy(ix.begin(), ix.end(), oix);
        *onnz = static_cast<int64_t>(ix.size());
        std::copy(e->map.begin(), e->map.end(), omap);
        std::copy(borders.begin(), borders.end(), oslices);
        *onslices = static_cast<int64_t>(borders.size());
        std::vector<int32_t> os, od;
        for (auto i : s) os.push_back(e->map[i]);
        for (auto i : d) od.push_back(e->map[i]);
        std::copy(os.begin(), os.end(), osrc);
        std::copy(od.begin(), od.end(), odest);
        auto find_offset = [&](std::vector<int32_t> const& idx) {
            int32_t const mx = *std::max_element(idx.begin(), idx.end());
            auto it = std::find_if(borders.begin(), borders.end(), [&](int32_t v) { return v > mx; });
            return static_cast<int64_t>(it - borders.begin());
        };
        offsets[0] = find_offset(os);
        offsets[1] = find_offset(od);
        e->map = saved_map;
    });
}

int kpm_set_progress_callback(kpm_engine* e, kpm_progress_fn fn, void* user) {
    return guarded([&] {
        if (!e) fail(KPM_ERR_VALUE, "null engine");
        HostThreads host_threads(e->cfg.num_threads);
        e->progress_fn = fn;
        e->progress_user = user;
    });
}

int kpm_get_stream(kpm_engine* e, void** stream) {
    return guarded([&] {
        if (!e || !stream) fail(KPM_ERR_VALUE, "null argument");
        e->ensure_device();
        *stream = static_cast<void*>(e->stream);
    });
}

int kpm_damping_coefficients(int32_t kernel, double param, int64_t M, double* out) {
    return guarded([&] {
        if (M < 0 || (M > 0 && !out)) fail(KPM_ERR_VALUE, "bad arguments");
        if (kernel == KPM_KERNEL_LORENTZ && param <= 0) fail(KPM_ERR_VALUE, "Lorentz kernel: lambda must be positive.");
        auto g = damping(kernel, param, M);
        std::copy(g.begin(), g.end(), out);
    });
}

int64_t kpm_required_num_moments(int32_t kernel, double param, double scaled_broadening) {
    return required_moments(kernel, param, scaled_broadening);
}

}  // extern "C"
