// KPM oracle: a CPU restatement of pybinding's kernel polynomial method.
//
// TEST INFRASTRUCTURE ONLY. This library is the checker for the GPU engine in
// pybinding_gb300/: only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline legs load it. The product never links, imports or calls it.
//
// Every routine restates the reference algorithm in the reference's own
// scalar type (float, double, complex<float>, complex<double>) and cites the
// reference file it follows (paths relative to the pybinding source tree).
// Random starters use libstdc++ <random> (std::mt19937, default seed 5489,
// std::uniform_real_distribution), the library the reference links on Linux,
// so the random vectors are the reference's bit for bit.
//
// Arrays cross the C ABI as plain pointers: complex values are interleaved
// (re, im) pairs of the real type; matrices of moments are column-major.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <mutex>
#include <numeric>
#include <random>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace orc {

template<class T> struct real_of { using type = T; };
template<class T> struct real_of<std::complex<T>> { using type = T; };
template<class T> using real_t = typename real_of<T>::type;
template<class T> struct is_cplx : std::false_type {};
template<class T> struct is_cplx<std::complex<T>> : std::true_type {};

// compute/detail.hpp:15-41
template<class R> inline R mul(R a, R b) { return a * b; }
template<class R> inline std::complex<R> mul(std::complex<R> a, std::complex<R> b) {
    return {a.real() * b.real() - a.imag() * b.imag(), a.real() * b.imag() + a.imag() * b.real()};
}
template<class R> inline R real_dot(R a, R b) { return a * b; }
template<class R> inline R real_dot(std::complex<R> a, std::complex<R> b) {
    return a.real() * b.real() + a.imag() * b.imag();
}
template<class R> inline R square(R a) { return a * a; }
template<class R> inline R square(std::complex<R> a) { return a.real() * a.real() + a.imag() * a.imag(); }
template<class R> inline R cj(R a) { return a; }
template<class R> inline std::complex<R> cj(std::complex<R> a) { return std::conj(a); }

template<class T> using Vec = std::vector<T>;

// Eigen's dot(): sum conj(a_i) b_i
template<class T> T dotc(T const* a, T const* b, int64_t start, int64_t end) {
    T s{0};
    for (auto i = start; i < end; ++i) s += mul(cj(a[i]), b[i]);
    return s;
}
template<class T> real_t<T> sqnorm(T const* a, int64_t start, int64_t end) {
    real_t<T> s{0};
    for (auto i = start; i < end; ++i) s += square(a[i]);
    return s;
}

template<class T>
struct CSR {
    int64_t rows = 0, cols = 0;
    Vec<int32_t> indptr, indices;
    Vec<T> values;
    int64_t nnz() const { return static_cast<int64_t>(values.size()); }
    bool empty() const { return rows == 0; }
};

template<class T>
CSR<T> csr_from(int64_t n, int32_t const* indptr, int32_t const* indices, void const* values) {
    CSR<T> m;
    m.rows = m.cols = n;
    m.indptr.assign(indptr, indptr + n + 1);
    auto const nnz = static_cast<int64_t>(indptr[n]);
    m.indices.assign(indices, indices + nnz);
    auto const v = static_cast<T const*>(values);
    m.values.assign(v, v + nnz);
    return m;
}

template<class T>
int64_t max_nnz_per_row(CSR<T> const& m) {
    int64_t r = 0;
    for (int64_t i = 0; i < m.rows; ++i) r = std::max<int64_t>(r, m.indptr[i + 1] - m.indptr[i]);
    return r;
}

// y = A x (Eigen sparse * dense, row-major)
template<class T>
Vec<T> csr_mv(CSR<T> const& a, Vec<T> const& x) {
    Vec<T> y(a.rows);
    for (int64_t r = 0; r < a.rows; ++r) {
        T s{0};
        for (auto n = a.indptr[r]; n < a.indptr[r + 1]; ++n) s += a.values[n] * x[a.indices[n]];
        y[r] = s;
    }
    return y;
}

// numeric/ellmatrix.hpp:11-82: column-major, rows padded to 32 bytes,
// padding value 0 with the previous row's column index.
template<class T>
struct Ell {
    int64_t rows = 0, width = 0, pitch_d = 0, pitch_i = 0;
    Vec<T> data;
    Vec<int32_t> indices;
    T& d(int64_t r, int64_t n) { return data[n * pitch_d + r]; }
    int32_t& i(int64_t r, int64_t n) { return indices[n * pitch_i + r]; }
    T const& d(int64_t r, int64_t n) const { return data[n * pitch_d + r]; }
    int32_t const& i(int64_t r, int64_t n) const { return indices[n * pitch_i + r]; }
};

inline int64_t aligned_size(int64_t rows, int64_t elem) {
    auto const per = 32 / elem;
    return per > 1 ? (rows + per - 1) / per * per : rows;
}

template<class T>
Ell<T> csr_to_ell(CSR<T> const& csr) {
    Ell<T> e;
    e.rows = csr.rows;
    e.width = max_nnz_per_row(csr);
    e.pitch_d = aligned_size(csr.rows, sizeof(T));
    e.pitch_i = aligned_size(csr.rows, sizeof(int32_t));
    e.data.assign(e.pitch_d * e.width, T{0});
    e.indices.assign(e.pitch_i * e.width, 0);
    for (int64_t r = 0; r < csr.rows; ++r) {
        int64_t n = 0;
        for (auto k = csr.indptr[r]; k < csr.indptr[r + 1]; ++k, ++n) {
            e.d(r, n) = csr.values[k];
            e.i(r, n) = csr.indices[k];
        }
        for (; n < e.width; ++n) {
            e.d(r, n) = T{0};
            e.i(r, n) = r > 0 ? e.i(r - 1, n) : 0;
        }
    }
    return e;
}

// ------------------------------------------------------------------ Scale, kpm/Bounds.hpp:11-37
struct Scale {
    double a = 0, b = 0;
};

inline Scale make_scale(double min_energy, double max_energy) {
    constexpr float tolerance = 0.01f;
    Scale s;
    s.a = 0.5f * (max_energy - min_energy) * (1 + tolerance);
    s.b = 0.5f * (max_energy + min_energy);
    if (std::abs(s.b / s.a) < 0.01f * tolerance) s.b = 0;
    return s;
}

// ------------------------------------------------------------------ kernels, kpm/Kernel.cpp:6-50
constexpr float PI_F = 3.14159265358979323846f;  // numeric/constant.hpp:7 (a float constant)

inline int64_t round_num_moments(int64_t n) {  // kpm/Kernel.hpp:9-13
    if (n < 2) return 2;
    while ((n - 2) % 4 != 0) ++n;
    return n;
}

enum KernelKind { JACKSON = 0, LORENTZ = 1, DIRICHLET = 2 };

inline Vec<double> damping(int kind, double lambda, int64_t num_moments) {
    Vec<double> g(num_moments);
    auto const N = static_cast<double>(num_moments);
    for (int64_t i = 0; i < num_moments; ++i) {
        auto const n = static_cast<double>(i);
        if (kind == JACKSON) {
            auto const Np = N + 1;
            constexpr double pi = double{PI_F};
            g[i] = ((Np - n) * std::cos(pi * n / Np) + std::sin(pi * n / Np) / std::tan(pi / Np)) / Np;
        } else if (kind == LORENTZ) {
            g[i] = std::sinh(lambda * (1 - n / N)) / std::sinh(lambda);
        } else {
            g[i] = 1.0;
        }
    }
    return g;
}

inline int64_t required_num_moments(int kind, double lambda, double scaled_broadening) {
    int64_t n;
    if (kind == LORENTZ) n = static_cast<int64_t>(lambda / scaled_broadening) + 1;
    else n = static_cast<int64_t>(PI_F / scaled_broadening) + 1;
    return round_num_moments(n);
}

// ------------------------------------------------------------------ Lanczos, compute/lanczos.hpp
template<class R>
void make_givens(R p, R q, R& c, R& s) {
    // Givens rotation G with G^T [p; q] = [r; 0] (the convention of Eigen's
    // JacobiRotation::makeGivens for real scalars).
    if (q == R(0)) {
        c = p < R(0) ? R(-1) : R(1);
        s = R(0);
    } else if (p == R(0)) {
        c = R(0);
        s = q < R(0) ? R(1) : R(-1);
    } else if (std::abs(p) > std::abs(q)) {
        R t = q / p;
        R u = std::sqrt(R(1) + t * t);
        if (p < R(0)) u = -u;
        c = R(1) / u;
        s = -t * c;
    } else {
        R t = p / q;
        R u = std::sqrt(R(1) + t * t);
        if (q < R(0)) u = -u;
        s = -R(1) / u;
        c = -t * s;
    }
}

// Implicit symmetric QR step with Wilkinson shift (compute/eigen3/lanczos.hpp:9-50)
template<class R>
void tridiagonal_qr_step(R* diag, R* subdiag, int start, int end) {
    R td = (diag[end - 1] - diag[end]) * R(0.5);
    R e = subdiag[end - 1];
    R mu = diag[end];
    if (td == R(0)) {
        mu -= std::abs(e);
    } else {
        R e2 = e * e;
        R h = std::hypot(td, e);
        if (e2 == R(0)) mu -= (e / (td + (td > 0 ? 1 : -1))) * (e / h);
        else mu -= e2 / (td + (td > 0 ? h : -h));
    }
    R x = diag[start] - mu;
    R z = subdiag[start];
    for (int k = start; k < end; ++k) {
        R c, s;
        make_givens(x, z, c, s);
        R sdk = s * diag[k] + c * subdiag[k];
        R dkp1 = s * subdiag[k] + c * diag[k + 1];
        diag[k] = c * (c * diag[k] - s * subdiag[k]) - s * (c * subdiag[k] - s * diag[k + 1]);
        diag[k + 1] = s * sdk + c * dkp1;
        subdiag[k] = c * sdk - s * dkp1;
        if (k > start) subdiag[k - 1] = c * subdiag[k - 1] - s * z;
        x = subdiag[k];
        if (k < end - 1) {
            z = -s * subdiag[k + 1];
            subdiag[k + 1] = c * subdiag[k + 1];
        }
    }
}

// compute/eigen3/lanczos.hpp:52-88
template<class R>
Vec<R> tridiagonal_eigenvalues(Vec<R> const& alpha, Vec<R> const& beta) {
    Vec<R> ev = alpha, tmp = beta;
    int start = 0;
    int end = static_cast<int>(ev.size()) - 1;
    int iter = 0;
    constexpr int max_iterations = 30;
    while (end > 0) {
        for (int i = start; i < end; ++i) {
            R a = std::abs(tmp[i]);
            R b = std::abs(ev[i]) + std::abs(ev[i + 1]);
            if (a < b * std::numeric_limits<R>::epsilon()) tmp[i] = 0;
        }
        while (end > 0 && tmp[end - 1] == R(0)) end--;
        if (end <= 0) break;
        if (++iter > max_iterations * static_cast<int>(ev.size()))
            throw std::runtime_error("Tridiagonal QR error");
        start = end - 1;
        while (start > 0 && tmp[start - 1] != R(0)) start--;
        tridiagonal_qr_step(ev.data(), tmp.data(), start, end);
    }
    return ev;
}

struct LanczosBounds { double min, max; int loops; };

// compute/lanczos.hpp:101-154
template<class T>
LanczosBounds minmax_eigenvalues(CSR<T> const& m, double precision_percent) {
    using R = real_t<T>;
    auto const n = m.rows;
    Vec<T> v0(n, T{0}), v1(n);
    {
        std::mt19937 gen;  // numeric/random.hpp:46-50: a fresh default-seeded generator
        std::uniform_real_distribution<R> dist;
        for (auto& v : v1) v = T(dist(gen));
        R nrm = std::sqrt(sqnorm(v1.data(), 0, n));
        if (nrm > R(0)) for (auto& v : v1) v = v / nrm;
    }
    Vec<R> alpha, beta;
    R prev_min = std::numeric_limits<R>::max();
    R prev_max = std::numeric_limits<R>::lowest();
    R const precision = static_cast<R>(precision_percent / 100);
    for (int i = 0; i < 1000; ++i) {
        R b_prev = beta.empty() ? R(0) : beta.back();
        R a{0};
        for (int64_t row = 0; row < n; ++row) {  // lanczos_spmv
            T t{0};
            for (auto k = m.indptr[row]; k < m.indptr[row + 1]; ++k) t += mul(m.values[k], v1[m.indices[k]]);
            v0[row] = t - b_prev * v0[row];
            a += real_dot(t, v1[row]);
        }
        R norm2{0};
        for (int64_t row = 0; row < n; ++row) {  // lanczos_axpy
            T l = v0[row] - a * v1[row];
            norm2 += square(l);
            v0[row] = l;
        }
        R b = std::sqrt(norm2);
        R inv = 1 / b;
        for (auto& v : v0) v *= inv;
        std::swap(v0, v1);
        alpha.push_back(a);
        beta.push_back(b);
        auto ev = tridiagonal_eigenvalues(alpha, beta);
        R mn = *std::min_element(ev.begin(), ev.end());
        R mx = *std::max_element(ev.begin(), ev.end());
        bool cmin = std::abs((prev_min - mn) / mn) < precision;
        bool cmax = std::abs((prev_max - mx) / mx) < precision;
        if (cmin && cmax) return {mn, mx, i};
        prev_min = mn;
        prev_max = mx;
    }
    throw std::runtime_error("Lanczos algorithm did not converge for the min/max eigenvalues.");
}

// ------------------------------------------------------------------ OptimizedHamiltonian
struct Indices {
    Vec<int32_t> src, dest;
    bool is_diagonal() const { return src.size() == dest.size() && src == dest; }
};

// kpm/OptimizedHamiltonian.hpp:54-96 + OptimizedHamiltonian.cpp:5-18
struct SliceMap {
    Vec<int32_t> data;
    int64_t src_offset = 0, dest_offset = 0;

    SliceMap() = default;
    explicit SliceMap(int64_t size) : data{static_cast<int32_t>(size)} {}
    SliceMap(Vec<int32_t> borders, Indices const& opt) : data(std::move(borders)) {
        auto find_offset = [&](Vec<int32_t> const& idx) {
            auto mx = *std::max_element(idx.begin(), idx.end());
            auto it = std::find_if(data.begin(), data.end(), [&](int32_t v) { return v > mx; });
            return static_cast<int64_t>(it - data.begin());
        };
        src_offset = find_offset(opt.src);
        dest_offset = find_offset(opt.dest);
    }
    int64_t last_index() const { return static_cast<int64_t>(data.size()) - 1; }
    int64_t index(int64_t n, int64_t M) const {
        auto const mid = (M - 1 + dest_offset - src_offset) / 2;
        auto const mx = std::min(last_index(), mid + src_offset);
        if (n < mid) return std::min(mx, n + src_offset);
        return std::min(mx, M - 1 - n + dest_offset);
    }
    int64_t optimal_size(int64_t n, int64_t M) const { return data[index(n, M)]; }
    int64_t operator[](int64_t i) const { return data[i]; }
};

template<class T>
struct Optimized {
    CSR<T> h2;
    Indices idx;
    SliceMap map;
    Vec<int32_t> reorder_map;  // empty when not reordered

    template<class V> void reorder(V& v) const {  // OptimizedHamiltonian.hpp:125-135
        if (reorder_map.empty()) return;
        V out(v.size());
        for (size_t i = 0; i < v.size(); ++i) out[reorder_map[i]] = v[i];
        v.swap(out);
    }
    void reorder(CSR<T>& m) const {  // OptimizedHamiltonian.hpp:137-151
        if (reorder_map.empty()) return;
        Vec<Vec<std::pair<int32_t, T>>> rows(m.rows);
        for (int64_t r = 0; r < m.rows; ++r)
            for (auto k = m.indptr[r]; k < m.indptr[r + 1]; ++k)
                rows[reorder_map[r]].push_back({reorder_map[m.indices[k]], m.values[k]});
        CSR<T> out;
        out.rows = m.rows;
        out.cols = m.cols;
        out.indptr.assign(m.rows + 1, 0);
        for (int64_t r = 0; r < m.rows; ++r) {
            std::sort(rows[r].begin(), rows[r].end(),
                      [](std::pair<int32_t, T> const& a, std::pair<int32_t, T> const& b) { return a.first < b.first; });
            for (auto& p : rows[r]) { out.indices.push_back(p.first); out.values.push_back(p.second); }
            out.indptr[r + 1] = static_cast<int32_t>(out.indices.size());
        }
        m = std::move(out);
    }
};

// OptimizedHamiltonian.cpp:55-72
template<class T>
Optimized<T> create_scaled(CSR<T> const& h, Indices const& idx, Scale s) {
    using R = real_t<T>;
    R const a = static_cast<R>(s.a), b = static_cast<R>(s.b);
    R const factor = 2 / a;
    Optimized<T> oh;
    auto& h2 = oh.h2;
    h2.rows = h2.cols = h.rows;
    h2.indptr.assign(h.rows + 1, 0);
    for (int64_t r = 0; r < h.rows; ++r) {
        bool diag_done = false;
        for (auto k = h.indptr[r]; k < h.indptr[r + 1]; ++k) {
            auto const c = h.indices[k];
            if (b != R(0) && !diag_done && c > r) {  // (H - I b) has a new diagonal entry here
                h2.indices.push_back(static_cast<int32_t>(r));
                h2.values.push_back((T(0) - T(b)) * factor);
                diag_done = true;
            }
            T v = h.values[k];
            if (b != R(0) && c == r) { v = v - T(b); diag_done = true; }
            h2.indices.push_back(c);
            h2.values.push_back(b != R(0) ? v * factor : h.values[k] * factor);
        }
        if (b != R(0) && !diag_done) {
            h2.indices.push_back(static_cast<int32_t>(r));
            h2.values.push_back((T(0) - T(b)) * factor);
        }
        h2.indptr[r + 1] = static_cast<int32_t>(h2.indices.size());
    }
    oh.idx = idx;
    oh.map = SliceMap(h.rows);
    return oh;
}

// OptimizedHamiltonian.cpp:75-152
template<class T>
Optimized<T> create_reordered(CSR<T> const& h, Indices const& idx, Scale s) {
    using R = real_t<T>;
    R const sa = static_cast<R>(s.a), sb = static_cast<R>(s.b);
    auto const n = h.rows;
    R const inverted_a = R{2 / sa};

    Optimized<T> oh;
    Vec<int32_t> queue;
    queue.reserve(n);
    queue.push_back(idx.src[0]);
    oh.reorder_map.assign(n, -1);
    oh.reorder_map[idx.src[0]] = 0;
    Vec<int32_t> borders{1};

    auto& h2 = oh.h2;
    h2.rows = h2.cols = n;
    h2.indptr.assign(n + 1, 0);
    Vec<std::pair<int32_t, T>> row_buf;
    int32_t next_unvisited = 0;
    for (int64_t h2_row = 0; h2_row < n; ++h2_row) {
        bool diagonal_inserted = false;
        if (h2_row == static_cast<int64_t>(queue.size())) {
            // disconnected graph: the reference reads past its queue here (it assumes a connected
            // system); continue from the first row not reached yet, as the engine does
            while (oh.reorder_map[next_unvisited] >= 0) ++next_unvisited;
            oh.reorder_map[next_unvisited] = static_cast<int32_t>(queue.size());
            queue.push_back(next_unvisited);
        }
        auto const row = queue[h2_row];
        row_buf.clear();
        for (auto k = h.indptr[row]; k < h.indptr[row + 1]; ++k) {
            auto const col = h.indices[k];
            if (oh.reorder_map[col] < 0) {
                oh.reorder_map[col] = static_cast<int32_t>(queue.size());
                queue.push_back(col);
            }
            auto const h2_col = oh.reorder_map[col];
            T v = h.values[k] * inverted_a;
            if (row == col) {
                v -= sb * inverted_a;
                diagonal_inserted = true;
            }
            row_buf.push_back({h2_col, v});
        }
        if (sb != R(0) && !diagonal_inserted) row_buf.push_back({static_cast<int32_t>(h2_row), T(-sb * inverted_a)});
        // Eigen's insert() into a reserved row keeps the inner indices sorted
        std::sort(row_buf.begin(), row_buf.end(),
                  [](std::pair<int32_t, T> const& a, std::pair<int32_t, T> const& b) { return a.first < b.first; });
        for (auto& p : row_buf) { h2.indices.push_back(p.first); h2.values.push_back(p.second); }
        h2.indptr[h2_row + 1] = static_cast<int32_t>(h2.indices.size());
        if (h2_row == borders.back() - 1) borders.push_back(static_cast<int32_t>(queue.size()));
    }
    borders.pop_back();
    Indices opt;
    for (auto i : idx.src) opt.src.push_back(oh.reorder_map[i]);
    for (auto i : idx.dest) opt.dest.push_back(oh.reorder_map[i]);
    oh.idx = opt;
    oh.map = SliceMap(std::move(borders), opt);
    return oh;
}

template<class T>
Optimized<T> optimize(CSR<T> const& h, Indices const& idx, Scale s, bool reorder) {
    return reorder ? create_reordered(h, idx, s) : create_scaled(h, idx, s);
}

// ------------------------------------------------------------------ SpMV, compute/kernel_polynomial.hpp
template<class T> struct Mat {  // either CSR or ELL view of the optimized matrix
    CSR<T> const* csr = nullptr;
    Ell<T> const* ell = nullptr;
    int64_t rows() const { return csr ? csr->rows : ell->rows; }
};

// y = H2 x - y over rows [start, end)   (kernel_polynomial.hpp:18-32, 88-118)
template<class T>
void kpm_spmv(int64_t start, int64_t end, Mat<T> const& m, T const* x, T* y) {
    if (m.csr) {
        auto const& a = *m.csr;
        for (auto row = start; row < end; ++row) {
            T r{0};
            for (auto n = a.indptr[row]; n < a.indptr[row + 1]; ++n) r += mul(a.values[n], x[a.indices[n]]);
            y[row] = r - y[row];
        }
    } else {
        auto const& e = *m.ell;
        for (auto row = start; row < end; ++row) y[row] = -y[row];
        for (int64_t n = 0; n < e.width; ++n)
            for (auto row = start; row < end; ++row) y[row] = mul(e.d(row, n), x[e.i(row, n)]) + y[row];
    }
}

// y = H2 x - y; m2 += |x|^2; m3 += <y|x>   (kernel_polynomial.hpp:60-81, 219-285)
template<class T>
void kpm_spmv_diagonal(int64_t start, int64_t end, Mat<T> const& m, T const* x, T* y, T& m2, T& m3) {
    kpm_spmv(start, end, m, x, y);
    m2 += T(sqnorm(x, start, end));
    m3 += dotc(y, x, start, end);
}

// Starter.hpp:55-118: r1 = 0.5 H2 r0
template<class T>
Vec<T> make_r1(Mat<T> const& m, Vec<T> const& r0) {
    auto const n = m.rows();
    Vec<T> r1(n, T{0});
    if (m.csr) {
        auto const& a = *m.csr;
        for (int64_t row = 0; row < n; ++row) {
            T t{0};
            for (auto k = a.indptr[row]; k < a.indptr[row + 1]; ++k) t += mul(a.values[k], r0[a.indices[k]]);
            r1[row] = t * T(0.5);
        }
    } else {
        auto const& e = *m.ell;
        for (int64_t k = 0; k < e.width; ++k)
            for (int64_t row = 0; row < n; ++row) r1[row] += mul(e.d(row, k), r0[e.i(row, k)]) * T(0.5);
    }
    return r1;
}

// ------------------------------------------------------------------ recursion drivers, kpm/calc_moments.hpp
// Diagonal collector, kpm/default/collectors.cpp:6-16
template<class T>
struct DiagCollect {
    Vec<T> moments;
    T m0{}, m1{};
    explicit DiagCollect(int64_t M) : moments(M, T{0}) {}
    void initial(Vec<T> const& r0, Vec<T> const& r1) {
        m0 = moments[0] = T(sqnorm(r0.data(), 0, static_cast<int64_t>(r0.size()))) * T(0.5);
        m1 = moments[1] = dotc(r1.data(), r0.data(), 0, static_cast<int64_t>(r0.size()));
    }
    void operator()(int64_t n, T m2, T m3) {
        moments[2 * (n - 1)] = T(2) * (m2 - m0);
        moments[2 * (n - 1) + 1] = T(2) * m3 - m1;
    }
};

template<class T>
void diag_basic(DiagCollect<T>& c, Vec<T> r0, Vec<T> r1, Mat<T> const& h2, SliceMap const& map, bool opt) {
    auto const M = static_cast<int64_t>(c.moments.size());
    for (int64_t n = 2; n <= M / 2; ++n) {
        T m2{0}, m3{0};
        auto const size = opt ? map.optimal_size(n, M) : h2.rows();
        kpm_spmv_diagonal<T>(0, size, h2, r1.data(), r0.data(), m2, m3);
        c(n, m2, m3);
        r1.swap(r0);
    }
}

template<class T>
void diag_interleaved(DiagCollect<T>& c, Vec<T> r0, Vec<T> r1, Mat<T> const& h2, SliceMap const& map, bool opt) {
    auto const M = static_cast<int64_t>(c.moments.size());
    if ((M - 2) % 4 != 0) throw std::logic_error("interleaved diagonal KPM needs (M - 2) % 4 == 0");
    for (int64_t n = 2; n <= M / 2; n += 2) {
        T m2{0}, m3{0}, m4{0}, m5{0};
        auto const max1 = opt ? map.index(n, M) : map.last_index();
        auto const max2 = opt ? map.index(n + 1, M) : map.last_index();
        for (int64_t k = 0, s0 = 0, s1 = 0; k <= max1; ++k) {
            auto const e0 = map[k];
            auto const e1 = (k == max1) ? map[max2] : s0;
            kpm_spmv_diagonal<T>(s0, e0, h2, r1.data(), r0.data(), m2, m3);
            kpm_spmv_diagonal<T>(s1, e1, h2, r0.data(), r1.data(), m4, m5);
            s1 = e1;
            s0 = e0;
        }
        c(n, m2, m3);
        c(n + 1, m4, m5);
    }
}

// Off-diagonal: collect(n, r) for n = 2 .. M-1   (calc_moments.hpp:102-146)
template<class T, class Collect>
void offdiag_basic(Collect&& collect, int64_t M, Vec<T> r0, Vec<T> r1, Mat<T> const& h2, SliceMap const& map, bool opt) {
    for (int64_t n = 2; n < M; ++n) {
        auto const size = opt ? map.optimal_size(n, M) : h2.rows();
        kpm_spmv<T>(0, size, h2, r1.data(), r0.data());
        r1.swap(r0);
        collect(n, r1);
    }
}

template<class T, class Collect>
void offdiag_interleaved(Collect&& collect, int64_t M, Vec<T> r0, Vec<T> r1, Mat<T> const& h2, SliceMap const& map, bool opt) {
    if (M % 2 != 0) throw std::logic_error("interleaved off-diagonal KPM needs an even M");
    for (int64_t n = 2; n < M; n += 2) {
        auto const max1 = opt ? map.index(n, M) : map.last_index();
        auto const max2 = opt ? map.index(n + 1, M) : map.last_index();
        for (int64_t k = 0, s0 = 0, s1 = 0; k <= max1; ++k) {
            auto const e0 = map[k];
            auto const e1 = (k == max1) ? map[max2] : s0;
            kpm_spmv<T>(s0, e0, h2, r1.data(), r0.data());
            kpm_spmv<T>(s1, e1, h2, r0.data(), r1.data());
            s1 = s0;
            s0 = e0;
        }
        collect(n, r0);
        collect(n + 1, r1);
    }
}

struct Algo { bool optimal_size = true, interleaved = true, ell = true; };

template<class T>
struct Engine {
    Optimized<T> oh;
    Ell<T> ell;
    bool use_ell;
    Mat<T> mat() const { Mat<T> m; if (use_ell) m.ell = &ell; else m.csr = &oh.h2; return m; }
    Engine(Optimized<T> o, bool ell_fmt) : oh(std::move(o)), use_ell(ell_fmt) {
        if (use_ell) ell = csr_to_ell(oh.h2);
    }

    // DefaultCompute::with + DiagonalCollector (default/Compute.cpp:24-44)
    Vec<T> diagonal(Vec<T> const& r0, int64_t M, Algo const& a) const {
        auto const m = mat();
        auto r1 = make_r1(m, r0);
        DiagCollect<T> c(M);
        c.initial(r0, r1);
        if (a.interleaved) diag_interleaved<T>(c, r0, r1, m, oh.map, a.optimal_size);
        else diag_basic<T>(c, r0, r1, m, oh.map, a.optimal_size);
        return c.moments;
    }

    template<class Init, class Collect>
    void offdiagonal(Vec<T> const& r0, int64_t M, Algo const& a, Init&& init, Collect&& collect) const {
        auto const m = mat();
        auto r1 = make_r1(m, r0);
        init(r0, r1);
        if (a.interleaved) offdiag_interleaved<T>(collect, M, r0, r1, m, oh.map, a.optimal_size);
        else offdiag_basic<T>(collect, M, r0, r1, m, oh.map, a.optimal_size);
    }
};

// ------------------------------------------------------------------ starters, kpm/Starter.cpp:48-84
template<class T>
struct RandomStarter {
    std::mt19937 gen;  // default seed 5489, one generator per starter
    CSR<T> op;         // optional operator in the original order
    Vec<T> make(int64_t n) {
        using R = real_t<T>;
        std::uniform_real_distribution<R> dist;
        Vec<T> r0(n);
        if constexpr (is_cplx<T>::value) {
            // k = complex<real_t>{2 * pi * i1}: built from the float constants
            std::complex<float> const kf = 2 * PI_F * std::complex<float>(0, 1);
            std::complex<R> const k(static_cast<R>(kf.real()), static_cast<R>(kf.imag()));
            for (int64_t i = 0; i < n; ++i) {
                R const phase = dist(gen);
                r0[i] = std::exp(k * phase);
            }
        } else {
            for (int64_t i = 0; i < n; ++i) r0[i] = (dist(gen) < 0.5f) ? R(-1.f) : R(1.f);
        }
        if (!op.empty()) r0 = csr_mv(op, r0);
        return r0;
    }
};

// velocity, kpm/Moments.cpp:132-155
template<class T>
CSR<T> velocity(CSR<T> const& h, float const* alpha) {
    auto v = h;
    for (int64_t row = 0; row < v.rows; ++row)
        for (auto n = v.indptr[row]; n < v.indptr[row + 1]; ++n)
            v.values[n] *= static_cast<T>(alpha[row] - alpha[v.indices[n]]);
    return v;
}

// ------------------------------------------------------------------ reconstruction, kpm/reconstruct.hpp
template<class R>
void spectral_density(Vec<std::complex<double>> const& moments_cd, int64_t M, int64_t cols,
                      double const* energy, int64_t ne, Scale s, double* out) {
    // moments_cd holds moments cast from the scalar type; only real parts are used
    R const a = static_cast<R>(s.a), b = static_cast<R>(s.b);
    R const k = R{2 / PI_F} / a;
    for (int64_t i = 0; i < ne; ++i) {
        R const E = (static_cast<R>(energy[i]) - b) / a;
        R const t = std::acos(E);
        for (int64_t c = 0; c < cols; ++c) {
            R sum{0};
            for (int64_t n = 0; n < M; ++n)
                sum += static_cast<R>(moments_cd[c * M + n].real()) * std::cos(static_cast<R>(n) * t);
            out[c * ne + i] = static_cast<double>(k / std::sqrt(1 - E * E) * sum);
        }
    }
}

template<class R>
void greens_function(Vec<std::complex<R>> const& moments, double const* energy, int64_t ne, Scale s,
                     double* out) {
    using C = std::complex<R>;
    R const a = static_cast<R>(s.a), b = static_cast<R>(s.b);
    C const i1 = C(std::complex<float>(0, 1));
    C const k = -R{2} * i1 / a;
    auto const M = static_cast<int64_t>(moments.size());
    for (int64_t i = 0; i < ne; ++i) {
        R const E = (static_cast<R>(energy[i]) - b) / a;
        R const t = std::acos(E);
        C sum{0};
        for (int64_t n = 0; n < M; ++n) sum += moments[n] * std::exp(-i1 * static_cast<R>(n) * t);
        C const g = k / std::sqrt(1 - E * E) * sum;
        out[2 * i] = static_cast<double>(g.real());
        out[2 * i + 1] = static_cast<double>(g.imag());
    }
}

// KuboBastin, reconstruct.hpp:90-143. mu is M x M column-major in the scalar type.
template<class T>
void kubo_bastin(Vec<T> const& mu, int64_t M, double const* chem, int64_t nchem,
                 double const* samples, int64_t ns, double temperature, Scale s, double* out) {
    using R = real_t<T>;
    using C = std::complex<R>;
    R const a = static_cast<R>(s.a), b = static_cast<R>(s.b);
    R const inv_kbt_sc = static_cast<R>(s.a / (8.6173303e-5f * temperature));
    C const i1 = C(std::complex<float>(0, 1));
    Vec<R> se(ns);
    for (int64_t i = 0; i < ns; ++i) se[i] = (static_cast<R>(samples[i]) - b) / a;
    R const coeff = (*std::max_element(se.begin(), se.end()) - *std::min_element(se.begin(), se.end()))
                    / static_cast<R>(2 * ns);
    Vec<C> sum_nm(ns);
    Vec<C> A(M);
    Vec<R> Tm(M);
    for (int64_t e = 0; e < ns; ++e) {
        R const en = se[e];
        R const sq = std::sqrt(R{1} - en * en);
        R const th = std::acos(en);
        for (int64_t n = 0; n < M; ++n) {
            R const nr = static_cast<R>(n);
            A[n] = (en - i1 * nr * sq) * std::exp(i1 * th * nr);
            Tm[n] = std::cos(th * nr);
        }
        // gamma[m][n] = A_n T_m + conj(A_m) T_n
        C acc{0};
        for (int64_t n = 0; n < M; ++n)
            for (int64_t m = 0; m < M; ++m) {
                C const g = A[n] * Tm[m] + std::conj(A[m]) * Tm[n];
                acc += C(mu[n * M + m]) * g;
            }
        R const k = R{1} / ((R{1} - en * en) * (R{1} - en * en));
        sum_nm[e] = k * acc;
    }
    C const prefix = C(T{4}) / (a * a);
    for (int64_t j = 0; j < nchem; ++j) {
        R const mu_s = (static_cast<R>(chem[j]) - b) / a;
        C total{0};
        for (int64_t e = 0; e < ns; ++e) {
            R const fd = R{1} / (R{1} + std::exp((se[e] - mu_s) * inv_kbt_sc));
            C const f = fd * sum_nm[e];
            total += (e == 0 || e == ns - 1) ? f : R{2} * f;
        }
        C const r = prefix * (coeff * total);
        out[2 * j] = static_cast<double>(r.real());
        out[2 * j + 1] = static_cast<double>(r.imag());
    }
}

// ------------------------------------------------------------------ Core, kpm/Core.cpp
struct Config {
    float min_energy = 0, max_energy = 0;
    int kernel = JACKSON;
    double lambda = 4.0;
    Algo algo;
    float lanczos_precision = 0.002f;
};

template<class T>
struct Core {
    CSR<T> h;
    Config cfg;
    double emin = 0, emax = 0;
    int loops = 0;
    bool have_bounds = false;

    Core(CSR<T> hh, Config c) : h(std::move(hh)), cfg(c) {
        if (cfg.min_energy > cfg.max_energy)
            throw std::invalid_argument("KPM: Invalid energy range specified (min > max).");
        if (cfg.min_energy != cfg.max_energy) {
            emin = cfg.min_energy; emax = cfg.max_energy; have_bounds = true;
        }
    }
    Scale scale() {
        if (!have_bounds) {
            auto lb = minmax_eigenvalues(h, static_cast<double>(cfg.lanczos_precision));
            emin = lb.min; emax = lb.max; loops = lb.loops; have_bounds = true;
        }
        return make_scale(emin, emax);
    }
    Algo no_opt() const { auto a = cfg.algo; a.optimal_size = false; return a; }
    bool reorder() const { return cfg.algo.optimal_size || cfg.algo.interleaved; }
    Engine<T> engine(Indices const& idx, Scale s) { return Engine<T>(optimize(h, idx, s, reorder()), cfg.algo.ell); }

    static Vec<std::complex<double>> to_cd(Vec<T> const& v) {
        Vec<std::complex<double>> r(v.size());
        for (size_t i = 0; i < v.size(); ++i) r[i] = std::complex<double>(v[i]);
        return r;
    }
    void damp(Vec<T>& m) const {
        auto g = damping(cfg.kernel, cfg.lambda, static_cast<int64_t>(m.size()));
        for (size_t i = 0; i < m.size(); ++i) m[i] *= static_cast<real_t<T>>(g[i]);
    }

    // Core::dos, Core.cpp:74-90
    void dos(double const* energy, int64_t ne, double broadening, int64_t num_random, double* out) {
        auto const s = scale();
        auto const M = required_num_moments(cfg.kernel, cfg.lambda, broadening / s.a);
        auto eng = engine(Indices{{0}, {0}}, s);
        RandomStarter<T> st;
        Vec<T> total(M, T{0});
        for (int64_t r = 0; r < num_random; ++r) {
            auto r0 = st.make(h.rows);
            eng.oh.reorder(r0);
            auto m = eng.diagonal(r0, M, no_opt());
            for (int64_t i = 0; i < M; ++i) total[i] += m[i];
        }
        if (num_random != 1)
            for (auto& v : total) v /= static_cast<real_t<T>>(num_random);
        damp(total);
        spectral_density<real_t<T>>(to_cd(total), M, 1, energy, ne, s, out);
    }

    // Core::ldos, Core.cpp:58-72 (out: ne x nidx column-major)
    void ldos(Vec<int32_t> const& idx, double const* energy, int64_t ne, double broadening, double* out) {
        auto const s = scale();
        auto const M = required_num_moments(cfg.kernel, cfg.lambda, broadening / s.a);
        auto eng = engine(Indices{idx, idx}, s);
        Vec<std::complex<double>> all;
        for (size_t i = 0; i < idx.size(); ++i) {
            Vec<T> r0(h.rows, T{0});
            r0[eng.oh.idx.src[i]] = T(1);
            auto m = eng.diagonal(r0, M, cfg.algo);
            damp(m);
            auto cd = to_cd(m);
            all.insert(all.end(), cd.begin(), cd.end());
        }
        spectral_density<real_t<T>>(all, M, static_cast<int64_t>(idx.size()), energy, ne, s, out);
    }

    // Core::greens_vector, Core.cpp:96-117 (out: ncols x ne complex)
    void greens(int32_t row, Vec<int32_t> const& cols, double const* energy, int64_t ne, double broadening, double* out) {
        using R = real_t<T>;
        auto const s = scale();
        auto const M = required_num_moments(cfg.kernel, cfg.lambda, broadening / s.a);
        Indices idx{{row}, cols};
        auto eng = engine(idx, s);
        Vec<T> r0(h.rows, T{0});
        r0[eng.oh.idx.src[0]] = T(1);
        Vec<Vec<T>> moments;
        if (idx.is_diagonal()) {
            moments.push_back(eng.diagonal(r0, M, cfg.algo));
        } else {
            auto const& dest = eng.oh.idx.dest;
            moments.assign(dest.size(), Vec<T>(M, T{0}));
            eng.offdiagonal(r0, M, cfg.algo,
                [&](Vec<T> const& a, Vec<T> const& b) {
                    for (size_t i = 0; i < dest.size(); ++i) {
                        moments[i][0] = a[dest[i]] * R{0.5};
                        moments[i][1] = b[dest[i]];
                    }
                },
                [&](int64_t n, Vec<T> const& r) { for (size_t i = 0; i < dest.size(); ++i) moments[i][n] = r[dest[i]]; });
        }
        for (size_t c = 0; c < moments.size(); ++c) {
            damp(moments[c]);
            Vec<std::complex<R>> m(M);
            for (int64_t i = 0; i < M; ++i) m[i] = std::complex<R>(moments[c][i]);
            greens_function<R>(m, energy, ne, s, out + 2 * ne * c);
        }
    }

    // Core::moments, Core.cpp:35-56 (alpha/beta complex double, op complex CSR)
    void moments(int64_t num_moments, Vec<T> alpha, Vec<T> beta, CSR<T> op, double* out) {
        auto const s = scale();
        auto const M = round_num_moments(num_moments);
        auto eng = engine(Indices{{0}, {0}}, s);
        eng.oh.reorder(alpha);
        Vec<T> m;
        if (beta.empty() && op.empty()) {
            m = eng.diagonal(alpha, M, no_opt());
        } else {
            // beta defaults to alpha (collectors.cpp:38-49); the caller passes it in the
            // original order, so it is reordered like the starter
            eng.oh.reorder(beta);
            if (!op.empty()) eng.oh.reorder(op);
            m.assign(M, T{0});
            auto apply = [&](Vec<T> const& r) { return op.empty() ? r : csr_mv(op, r); };
            auto const n = static_cast<int64_t>(alpha.size());
            eng.offdiagonal(alpha, M, no_opt(),
                [&](Vec<T> const& a, Vec<T> const& b) {
                    m[0] = dotc(beta.data(), apply(a).data(), 0, n);
                    m[0] *= 0.5f;
                    m[1] = dotc(beta.data(), apply(b).data(), 0, n);
                },
                [&](int64_t k, Vec<T> const& r) { m[k] = dotc(beta.data(), apply(r).data(), 0, n); });
        }
        damp(m);
        for (int64_t i = 0; i < num_moments; ++i) {
            std::complex<double> v(m[i]);
            out[2 * i] = v.real();
            out[2 * i + 1] = v.imag();
        }
    }

    // Core::conductivity, Core.cpp:119-150 (out: nchem complex)
    void conductivity(float const* left, float const* right, double const* chem, int64_t nchem,
                      double broadening, double temperature, int64_t num_random, int64_t num_points, double* out) {
        auto const s = scale();
        auto const M = required_num_moments(cfg.kernel, cfg.lambda, broadening / s.a);
        auto eng = engine(Indices{{0}, {0}}, s);
        auto const n = h.rows;
        RandomStarter<T> st_l, st_r;
        st_l.op = velocity(h, left);
        auto vr = velocity(h, right);
        eng.oh.reorder(vr);
        Vec<T> mu(M * M, T{0});
        Vec<T> L(M * n), Rm(M * n);  // row-major M x n
        for (int64_t j = 0; j < num_random; ++j) {
            auto rl = st_l.make(n);
            eng.oh.reorder(rl);
            eng.offdiagonal(rl, M, no_opt(),
                [&](Vec<T> const& a, Vec<T> const& b) {
                    for (int64_t i = 0; i < n; ++i) { L[i] = a[i] * real_t<T>(0.5); L[n + i] = b[i]; }
                },
                [&](int64_t k, Vec<T> const& r) { std::copy(r.begin(), r.end(), L.begin() + k * n); });
            auto rr = st_r.make(n);
            eng.oh.reorder(rr);
            eng.offdiagonal(rr, M, no_opt(),
                [&](Vec<T> const& a, Vec<T> const& b) {
                    auto va = csr_mv(vr, a), vb = csr_mv(vr, b);
                    for (int64_t i = 0; i < n; ++i) { Rm[i] = va[i] * real_t<T>(0.5); Rm[n + i] = vb[i]; }
                },
                [&](int64_t k, Vec<T> const& r) { auto v = csr_mv(vr, r); std::copy(v.begin(), v.end(), Rm.begin() + k * n); });
            // mu += L * R^H  (Moments.cpp:92-101)
            for (int64_t c = 0; c < M; ++c)
                for (int64_t r = 0; r < M; ++r) {
                    T acc{0};
                    T const* lr = L.data() + r * n;
                    T const* rc = Rm.data() + c * n;
                    for (int64_t i = 0; i < n; ++i) acc += lr[i] * cj(rc[i]);
                    mu[c * M + r] += acc;
                }
        }
        for (auto& v : mu) v /= static_cast<real_t<T>>(num_random);
        auto g = damping(cfg.kernel, cfg.lambda, M);
        for (int64_t c = 0; c < M; ++c)
            for (int64_t r = 0; r < M; ++r)
                mu[c * M + r] *= static_cast<real_t<T>>(g[r]) * static_cast<real_t<T>>(g[c]);
        Vec<double> samples(num_points);
        double const lo = emin, hi = emax;
        for (int64_t i = 0; i < num_points; ++i)
            samples[i] = num_points > 1 ? lo + (hi - lo) * static_cast<double>(i) / static_cast<double>(num_points - 1) : hi;
        if (num_points > 1) samples[num_points - 1] = hi;
        kubo_bastin<T>(mu, M, chem, nchem, samples.data(), num_points, temperature, s, out);
    }
};

// ------------------------------------------------------------------ CPU baseline (timed)
// Multithreaded restatement of DefaultCompute's DOS batches (default/Compute.cpp:52-88):
// ELL matrix, interleaved diagonal recursion, k vectors per batch stored
// row-major (vectors interleaved per row, like Eigen's row-major batch),
// one std::thread per core pulling batches from a shared counter.
// KC > 0 fixes the batch width at compile time (the reference's batches are SIMD-register
// wide, support/simd.hpp:35-43), so that the per-row loops over the batch vectorise fully.
template<class T, int KC>
void batch_interleaved(Ell<T> const& e, SliceMap const& map, T const* r0_in, int64_t k_runtime, int64_t M,
                       T* mu_out) {
    int64_t const k = KC > 0 ? KC : k_runtime;
    auto const n = e.rows;
    Vec<T> r0(r0_in, r0_in + n * k), r1(n * k, T{0});
    for (int64_t c = 0; c < e.width; ++c)
        for (int64_t row = 0; row < n; ++row) {
            auto const a = e.d(row, c) * T(0.5);
            T const* x = &r0[static_cast<int64_t>(e.i(row, c)) * k];
            T* y = &r1[row * k];
            for (int64_t j = 0; j < k; ++j) y[j] += a * x[j];
        }
    Vec<T> m0(k), m1(k);
    for (int64_t j = 0; j < k; ++j) { m0[j] = T{0}; m1[j] = T{0}; }
    for (int64_t row = 0; row < n; ++row)
        for (int64_t j = 0; j < k; ++j) {
            m0[j] += T(square(r0[row * k + j]));
            m1[j] += cj(r1[row * k + j]) * r0[row * k + j];
        }
    for (int64_t j = 0; j < k; ++j) {
        m0[j] *= T(0.5);
        mu_out[j * M + 0] = m0[j];
        mu_out[j * M + 1] = m1[j];
    }
    auto step = [&](int64_t s, int64_t t, T const* x, T* y, T* m2, T* m3) {
        for (int64_t c = 0; c < e.width; ++c) {
            for (int64_t row = s; row < t; ++row) {
                auto const a = e.d(row, c);
                T const* xr = x + static_cast<int64_t>(e.i(row, c)) * k;
                T* yr = y + row * k;
                if (c == 0) for (int64_t j = 0; j < k; ++j) yr[j] = a * xr[j] - yr[j];
                else for (int64_t j = 0; j < k; ++j) yr[j] += a * xr[j];
            }
        }
        for (int64_t row = s; row < t; ++row)
            for (int64_t j = 0; j < k; ++j) {
                m2[j] += T(square(x[row * k + j]));
                m3[j] += cj(y[row * k + j]) * x[row * k + j];
            }
    };
    Vec<T> m2(k), m3(k), m4(k), m5(k);
    for (int64_t nn = 2; nn <= M / 2; nn += 2) {
        std::fill(m2.begin(), m2.end(), T{0}); std::fill(m3.begin(), m3.end(), T{0});
        std::fill(m4.begin(), m4.end(), T{0}); std::fill(m5.begin(), m5.end(), T{0});
        auto const max1 = map.last_index();
        for (int64_t kk = 0, s0 = 0, s1 = 0; kk <= max1; ++kk) {
            auto const e0 = map[kk];
            auto const e1 = (kk == max1) ? map[max1] : s0;
            step(s0, e0, r1.data(), r0.data(), m2.data(), m3.data());
            step(s1, e1, r0.data(), r1.data(), m4.data(), m5.data());
            s1 = e1;
            s0 = e0;
        }
        for (int64_t j = 0; j < k; ++j) {
            mu_out[j * M + 2 * (nn - 1)] = T(2) * (m2[j] - m0[j]);
            mu_out[j * M + 2 * (nn - 1) + 1] = T(2) * m3[j] - m1[j];
            if (nn + 1 <= M / 2) {
                mu_out[j * M + 2 * nn] = T(2) * (m4[j] - m0[j]);
                mu_out[j * M + 2 * nn + 1] = T(2) * m5[j] - m1[j];
            }
        }
    }
}

template<class T>
void batch_any_width(Ell<T> const& e, SliceMap const& map, T const* r0, int64_t k, int64_t M, T* mu_out) {
    switch (k) {
        case 1: batch_interleaved<T, 1>(e, map, r0, k, M, mu_out); break;
        case 2: batch_interleaved<T, 2>(e, map, r0, k, M, mu_out); break;
        case 4: batch_interleaved<T, 4>(e, map, r0, k, M, mu_out); break;
        case 8: batch_interleaved<T, 8>(e, map, r0, k, M, mu_out); break;
        case 16: batch_interleaved<T, 16>(e, map, r0, k, M, mu_out); break;
        default: batch_interleaved<T, 0>(e, map, r0, k, M, mu_out); break;
    }
}

}  // namespace orc

// ====================================================================== C ABI
using namespace orc;

static thread_local std::string g_err;

template<class F>
static int guarded(F&& f) {
    try {
        f();
        return 0;
    } catch (std::invalid_argument const& e) {
        g_err = e.what();
        return 2;
    } catch (std::exception const& e) {
        g_err = e.what();
        return 1;
    }
}

template<template<class> class F, class... Args>
static void dispatch(int dtype, Args&&... args) {
    switch (dtype) {
        case 0: F<float>::run(std::forward<Args>(args)...); break;
        case 1: F<double>::run(std::forward<Args>(args)...); break;
        case 2: F<std::complex<float>>::run(std::forward<Args>(args)...); break;
        case 3: F<std::complex<double>>::run(std::forward<Args>(args)...); break;
        default: throw std::invalid_argument("unknown dtype code");
    }
}

struct OrcConfig {
    double min_energy, max_energy;
    int32_t kernel;
    double lambda;
    int32_t optimal_size, interleaved, ell;
    double lanczos_precision;
};

static Config to_cfg(OrcConfig const* c) {
    Config cfg;
    cfg.min_energy = static_cast<float>(c->min_energy);
    cfg.max_energy = static_cast<float>(c->max_energy);
    cfg.kernel = c->kernel;
    cfg.lambda = c->lambda;
    cfg.algo.optimal_size = c->optimal_size != 0;
    cfg.algo.interleaved = c->interleaved != 0;
    cfg.algo.ell = c->ell != 0;
    cfg.lanczos_precision = static_cast<float>(c->lanczos_precision);
    return cfg;
}

template<class T>
static Vec<T> from_cd(double const* v, int64_t n) {
    Vec<T> out(n);
    for (int64_t i = 0; i < n; ++i) {
        if constexpr (is_cplx<T>::value) out[i] = T(static_cast<real_t<T>>(v[2 * i]), static_cast<real_t<T>>(v[2 * i + 1]));
        else out[i] = static_cast<T>(v[2 * i]);
    }
    return out;
}

extern "C" const char* orc_last_error() { return g_err.c_str(); }

extern "C" void orc_scale(double emin, double emax, double* a, double* b) {
    auto s = make_scale(emin, emax);
    *a = s.a;
    *b = s.b;
}

extern "C" int64_t orc_round_num_moments(int64_t n) { return round_num_moments(n); }

extern "C" int64_t orc_required_num_moments(int32_t kernel, double lambda, double scaled_broadening) {
    return required_num_moments(kernel, lambda, scaled_broadening);
}

extern "C" void orc_damping(int32_t kernel, double lambda, int64_t n, double* out) {
    auto g = damping(kernel, lambda, n);
    std::copy(g.begin(), g.end(), out);
}

template<class T> struct LanczosF {
    static void run(int64_t n, int32_t const* ip, int32_t const* ix, void const* v, double prec,
                    double* mn, double* mx, int32_t* loops) {
        auto m = csr_from<T>(n, ip, ix, v);
        auto r = minmax_eigenvalues(m, prec);
        *mn = r.min; *mx = r.max; *loops = r.loops;
    }
};
extern "C" int orc_lanczos(int32_t dtype, int64_t n, int32_t const* ip, int32_t const* ix, void const* v,
                double precision_percent, double* mn, double* mx, int32_t* loops) {
    return guarded([&] { dispatch<LanczosF>(dtype, n, ip, ix, v, precision_percent, mn, mx, loops); });
}

// Optimize (reorder/scale) a CSR. Output buffers: indptr n+1, indices/values nnz+n,
// map n, slices n+1, src nsrc, dest ndest.
template<class T> struct OptimizeF {
    static void run(int64_t n, int32_t const* ip, int32_t const* ix, void const* v,
                    int32_t const* src, int64_t nsrc, int32_t const* dest, int64_t ndest,
                    double a, double b, int32_t reorder,
                    int32_t* oip, int32_t* oix, void* ov, int64_t* onnz, int32_t* omap,
                    int32_t* oslices, int64_t* onslices, int32_t* osrc, int32_t* odest,
                    int64_t* src_off, int64_t* dest_off) {
        auto m = csr_from<T>(n, ip, ix, v);
        Indices idx{Vec<int32_t>(src, src + nsrc), Vec<int32_t>(dest, dest + ndest)};
        Scale s{a, b};
        auto oh = optimize(m, idx, s, reorder != 0);
        std::copy(oh.h2.indptr.begin(), oh.h2.indptr.end(), oip);
        std::copy(oh.h2.indices.begin(), oh.h2.indices.end(), oix);
        std::copy(oh.h2.values.begin(), oh.h2.values.end(), static_cast<T*>(ov));
        *onnz = oh.h2.nnz();
        if (!oh.reorder_map.empty()) std::copy(oh.reorder_map.begin(), oh.reorder_map.end(), omap);
        else for (int64_t i = 0; i < n; ++i) omap[i] = static_cast<int32_t>(i);
        std::copy(oh.map.data.begin(), oh.map.data.end(), oslices);
        *onslices = static_cast<int64_t>(oh.map.data.size());
        std::copy(oh.idx.src.begin(), oh.idx.src.end(), osrc);
        std::copy(oh.idx.dest.begin(), oh.idx.dest.end(), odest);
        *src_off = oh.map.src_offset;
        *dest_off = oh.map.dest_offset;
    }
};
extern "C" int orc_optimize(int32_t dtype, int64_t n, int32_t const* ip, int32_t const* ix, void const* v,
                 int32_t const* src, int64_t nsrc, int32_t const* dest, int64_t ndest,
                 double a, double b, int32_t reorder,
                 int32_t* oip, int32_t* oix, void* ov, int64_t* onnz, int32_t* omap,
                 int32_t* oslices, int64_t* onslices, int32_t* osrc, int32_t* odest,
                 int64_t* src_off, int64_t* dest_off) {
    return guarded([&] {
        dispatch<OptimizeF>(dtype, n, ip, ix, v, src, nsrc, dest, ndest, a, b, reorder, oip, oix, ov,
                            onnz, omap, oslices, onslices, osrc, odest, src_off, dest_off);
    });
}

extern "C" int64_t orc_slicemap_index(int32_t const* slices, int64_t nslices, int64_t src_off, int64_t dest_off,
                           int64_t n, int64_t M) {
    SliceMap m;
    m.data.assign(slices, slices + nslices);
    m.src_offset = src_off;
    m.dest_offset = dest_off;
    return m.index(n, M);
}

// `count` random starter vectors in draw order from one fresh generator, original
// site order (not reordered), optional operator applied. out: count x n.
template<class T> struct StarterF {
    static void run(int64_t n, int64_t count, int64_t op_n, int32_t const* op_ip, int32_t const* op_ix,
                    void const* op_v, void* out) {
        RandomStarter<T> st;
        if (op_n > 0) st.op = csr_from<T>(op_n, op_ip, op_ix, op_v);
        auto o = static_cast<T*>(out);
        for (int64_t c = 0; c < count; ++c) {
            auto r = st.make(n);
            std::copy(r.begin(), r.end(), o + c * n);
        }
    }
};
extern "C" int orc_random_starters(int32_t dtype, int64_t n, int64_t count, int64_t op_n, int32_t const* op_ip,
                        int32_t const* op_ix, void const* op_v, void* out) {
    return guarded([&] { dispatch<StarterF>(dtype, n, count, op_n, op_ip, op_ix, op_v, out); });
}

// Diagonal moments on an already optimized (scaled/reordered) matrix for k starters
// given in that matrix's order. r0: k x n; out: k x M (scalar type).
template<class T> struct DiagF {
    static void run(int64_t n, int32_t const* ip, int32_t const* ix, void const* v,
                    int32_t const* slices, int64_t nslices, int64_t src_off, int64_t dest_off,
                    int32_t ell, int32_t opt_size, int32_t interleaved,
                    void const* r0, int64_t k, int64_t M, void* out) {
        Optimized<T> oh;
        oh.h2 = csr_from<T>(n, ip, ix, v);
        oh.map.data.assign(slices, slices + nslices);
        oh.map.src_offset = src_off;
        oh.map.dest_offset = dest_off;
        Engine<T> eng(std::move(oh), ell != 0);
        Algo a;
        a.optimal_size = opt_size != 0;
        a.interleaved = interleaved != 0;
        a.ell = ell != 0;
        auto rr = static_cast<T const*>(r0);
        auto o = static_cast<T*>(out);
        for (int64_t c = 0; c < k; ++c) {
            Vec<T> r(rr + c * n, rr + (c + 1) * n);
            auto m = eng.diagonal(r, M, a);
            std::copy(m.begin(), m.end(), o + c * M);
        }
    }
};
extern "C" int orc_moments_diag(int32_t dtype, int64_t n, int32_t const* ip, int32_t const* ix, void const* v,
                     int32_t const* slices, int64_t nslices, int64_t src_off, int64_t dest_off,
                     int32_t ell, int32_t opt_size, int32_t interleaved,
                     void const* r0, int64_t k, int64_t M, void* out) {
    return guarded([&] {
        dispatch<DiagF>(dtype, n, ip, ix, v, slices, nslices, src_off, dest_off, ell, opt_size, interleaved, r0, k, M, out);
    });
}

// Off-diagonal moments mu_n = <beta| T_n(H2/2) |r0> on an optimized matrix (no operator).
// out: M values (scalar type).
template<class T> struct OffF {
    static void run(int64_t n, int32_t const* ip, int32_t const* ix, void const* v, int32_t ell,
                    int32_t interleaved, void const* r0, void const* beta, int64_t M, void* out) {
        Optimized<T> oh;
        oh.h2 = csr_from<T>(n, ip, ix, v);
        oh.map = SliceMap(n);
        Engine<T> eng(std::move(oh), ell != 0);
        Algo a;
        a.optimal_size = false;
        a.interleaved = interleaved != 0;
        Vec<T> r(static_cast<T const*>(r0), static_cast<T const*>(r0) + n);
        Vec<T> bta(static_cast<T const*>(beta), static_cast<T const*>(beta) + n);
        auto o = static_cast<T*>(out);
        eng.offdiagonal(r, M, a,
            [&](Vec<T> const& x, Vec<T> const& y) {
                o[0] = dotc(bta.data(), x.data(), 0, n) * T(0.5f);
                o[1] = dotc(bta.data(), y.data(), 0, n);
            },
            [&](int64_t k, Vec<T> const& x) { o[k] = dotc(bta.data(), x.data(), 0, n); });
    }
};
extern "C" int orc_moments_offdiag(int32_t dtype, int64_t n, int32_t const* ip, int32_t const* ix, void const* v,
                        int32_t ell, int32_t interleaved, void const* r0, void const* beta, int64_t M, void* out) {
    return guarded([&] { dispatch<OffF>(dtype, n, ip, ix, v, ell, interleaved, r0, beta, M, out); });
}

// Dense matrix of vectors: row k = T_k(H2/2) r0 (row 0 halved), out: M x n row-major.
template<class T> struct DenseF {
    static void run(int64_t n, int32_t const* ip, int32_t const* ix, void const* v, void const* r0, int64_t M, void* out) {
        Optimized<T> oh;
        oh.h2 = csr_from<T>(n, ip, ix, v);
        oh.map = SliceMap(n);
        Engine<T> eng(std::move(oh), false);
        Algo a;
        a.optimal_size = false;
        a.interleaved = false;
        Vec<T> r(static_cast<T const*>(r0), static_cast<T const*>(r0) + n);
        auto o = static_cast<T*>(out);
        eng.offdiagonal(r, M, a,
            [&](Vec<T> const& x, Vec<T> const& y) {
                for (int64_t i = 0; i < n; ++i) { o[i] = x[i] * real_t<T>(0.5); o[n + i] = y[i]; }
            },
            [&](int64_t k, Vec<T> const& x) { std::copy(x.begin(), x.end(), o + k * n); });
    }
};
extern "C" int orc_dense_vectors(int32_t dtype, int64_t n, int32_t const* ip, int32_t const* ix, void const* v,
                      void const* r0, int64_t M, void* out) {
    return guarded([&] { dispatch<DenseF>(dtype, n, ip, ix, v, r0, M, out); });
}

template<class T> struct VelF {
    static void run(int64_t n, int32_t const* ip, int32_t const* ix, void const* v, float const* alpha, void* out) {
        auto m = csr_from<T>(n, ip, ix, v);
        auto r = velocity(m, alpha);
        std::copy(r.values.begin(), r.values.end(), static_cast<T*>(out));
    }
};
extern "C" int orc_velocity(int32_t dtype, int64_t n, int32_t const* ip, int32_t const* ix, void const* v,
                 float const* alpha, void* out) {
    return guarded([&] { dispatch<VelF>(dtype, n, ip, ix, v, alpha, out); });
}

// Reconstruction in the real type of `dtype` from complex-double moments.
extern "C" int orc_spectral_density(int32_t dtype, double const* moments, int64_t M, int64_t cols,
                         double const* energy, int64_t ne, double a, double b, double* out) {
    return guarded([&] {
        Vec<std::complex<double>> m(M * cols);
        for (int64_t i = 0; i < M * cols; ++i) m[i] = {moments[2 * i], moments[2 * i + 1]};
        Scale s{a, b};
        if (dtype == 0 || dtype == 2) spectral_density<float>(m, M, cols, energy, ne, s, out);
        else spectral_density<double>(m, M, cols, energy, ne, s, out);
    });
}

extern "C" int orc_greens_function(int32_t dtype, double const* moments, int64_t M, double const* energy, int64_t ne,
                        double a, double b, double* out) {
    return guarded([&] {
        Scale s{a, b};
        if (dtype == 0 || dtype == 2) {
            Vec<std::complex<float>> m(M);
            for (int64_t i = 0; i < M; ++i) m[i] = {static_cast<float>(moments[2 * i]), static_cast<float>(moments[2 * i + 1])};
            greens_function<float>(m, energy, ne, s, out);
        } else {
            Vec<std::complex<double>> m(M);
            for (int64_t i = 0; i < M; ++i) m[i] = {moments[2 * i], moments[2 * i + 1]};
            greens_function<double>(m, energy, ne, s, out);
        }
    });
}

extern "C" int orc_kubo_bastin(int32_t dtype, double const* mu, int64_t M, double const* chem, int64_t nchem,
                    double const* samples, int64_t ns, double temperature, double a, double b, double* out) {
    return guarded([&] {
        Scale s{a, b};
        if (dtype == 0 || dtype == 2) {
            Vec<std::complex<float>> m(M * M);
            for (int64_t i = 0; i < M * M; ++i) m[i] = {static_cast<float>(mu[2 * i]), static_cast<float>(mu[2 * i + 1])};
            kubo_bastin<std::complex<float>>(m, M, chem, nchem, samples, ns, temperature, s, out);
        } else {
            Vec<std::complex<double>> m(M * M);
            for (int64_t i = 0; i < M * M; ++i) m[i] = {mu[2 * i], mu[2 * i + 1]};
            kubo_bastin<std::complex<double>>(m, M, chem, nchem, samples, ns, temperature, s, out);
        }
    });
}

// ---- Core-level calls (the whole reference flow: Lanczos, reorder, starters, recursion,
// damping, reconstruction), used to pin the restatement against the reference goldens.
template<class T> struct CoreDosF {
    static void run(int64_t n, int32_t const* ip, int32_t const* ix, void const* v, OrcConfig const* c,
                    double const* energy, int64_t ne, double broadening, int64_t num_random, double* out, double* ab) {
        Core<T> core(csr_from<T>(n, ip, ix, v), to_cfg(c));
        core.dos(energy, ne, broadening, num_random, out);
        auto s = core.scale();
        ab[0] = s.a; ab[1] = s.b; ab[2] = core.emin; ab[3] = core.emax;
    }
};
extern "C" int orc_core_dos(int32_t dtype, int64_t n, int32_t const* ip, int32_t const* ix, void const* v, OrcConfig const* c,
                 double const* energy, int64_t ne, double broadening, int64_t num_random, double* out, double* ab) {
    return guarded([&] { dispatch<CoreDosF>(dtype, n, ip, ix, v, c, energy, ne, broadening, num_random, out, ab); });
}

template<class T> struct CoreLdosF {
    static void run(int64_t n, int32_t const* ip, int32_t const* ix, void const* v, OrcConfig const* c,
                    int32_t const* idx, int64_t nidx, double const* energy, int64_t ne, double broadening, double* out) {
        Core<T> core(csr_from<T>(n, ip, ix, v), to_cfg(c));
        core.ldos(Vec<int32_t>(idx, idx + nidx), energy, ne, broadening, out);
    }
};
extern "C" int orc_core_ldos(int32_t dtype, int64_t n, int32_t const* ip, int32_t const* ix, void const* v, OrcConfig const* c,
                  int32_t const* idx, int64_t nidx, double const* energy, int64_t ne, double broadening, double* out) {
    return guarded([&] { dispatch<CoreLdosF>(dtype, n, ip, ix, v, c, idx, nidx, energy, ne, broadening, out); });
}

template<class T> struct CoreGreensF {
    static void run(int64_t n, int32_t const* ip, int32_t const* ix, void const* v, OrcConfig const* c,
                    int32_t row, int32_t const* cols, int64_t ncols, double const* energy, int64_t ne,
                    double broadening, double* out) {
        Core<T> core(csr_from<T>(n, ip, ix, v), to_cfg(c));
        core.greens(row, Vec<int32_t>(cols, cols + ncols), energy, ne, broadening, out);
    }
};
extern "C" int orc_core_greens(int32_t dtype, int64_t n, int32_t const* ip, int32_t const* ix, void const* v, OrcConfig const* c,
                    int32_t row, int32_t const* cols, int64_t ncols, double const* energy, int64_t ne,
                    double broadening, double* out) {
    return guarded([&] { dispatch<CoreGreensF>(dtype, n, ip, ix, v, c, row, cols, ncols, energy, ne, broadening, out); });
}

template<class T> struct CoreMomentsF {
    static void run(int64_t n, int32_t const* ip, int32_t const* ix, void const* v, OrcConfig const* c,
                    int64_t num_moments, double const* alpha, double const* beta, int64_t op_n, int32_t const* op_ip,
                    int32_t const* op_ix, double const* op_v, double* out) {
        Core<T> core(csr_from<T>(n, ip, ix, v), to_cfg(c));
        Vec<T> a = from_cd<T>(alpha, n);
        Vec<T> b = beta ? from_cd<T>(beta, n) : (Vec<T>{});
        CSR<T> op;
        if (op_n > 0) {
            op.rows = op.cols = op_n;
            op.indptr.assign(op_ip, op_ip + op_n + 1);
            op.indices.assign(op_ix, op_ix + op_ip[op_n]);
            op.values = from_cd<T>(op_v, op_ip[op_n]);
        }
        if (b.empty() && !op.empty()) b = a;  // alpha doubles as beta
        core.moments(num_moments, a, b, op, out);
    }
};
extern "C" int orc_core_moments(int32_t dtype, int64_t n, int32_t const* ip, int32_t const* ix, void const* v, OrcConfig const* c,
                     int64_t num_moments, double const* alpha, double const* beta, int64_t op_n, int32_t const* op_ip,
                     int32_t const* op_ix, double const* op_v, double* out) {
    return guarded([&] {
        dispatch<CoreMomentsF>(dtype, n, ip, ix, v, c, num_moments, alpha, beta, op_n, op_ip, op_ix, op_v, out);
    });
}

template<class T> struct CoreCondF {
    static void run(int64_t n, int32_t const* ip, int32_t const* ix, void const* v, OrcConfig const* c,
                    float const* left, float const* right, double const* chem, int64_t nchem, double broadening,
                    double temperature, int64_t num_random, int64_t num_points, double* out) {
        Core<T> core(csr_from<T>(n, ip, ix, v), to_cfg(c));
        core.conductivity(left, right, chem, nchem, broadening, temperature, num_random, num_points, out);
    }
};
extern "C" int orc_core_conductivity(int32_t dtype, int64_t n, int32_t const* ip, int32_t const* ix, void const* v,
                          OrcConfig const* c, float const* left, float const* right, double const* chem, int64_t nchem,
                          double broadening, double temperature, int64_t num_random, int64_t num_points, double* out) {
    return guarded([&] {
        dispatch<CoreCondF>(dtype, n, ip, ix, v, c, left, right, chem, nchem, broadening, temperature, num_random,
                            num_points, out);
    });
}

// Timed CPU baseline: R starters (count x n, reordered already) over an optimized CSR,
// batches of k vectors, `threads` workers. mu_out: R x M (scalar type). Returns seconds.
template<class T> struct BenchF {
    static void run(int64_t n, int32_t const* ip, int32_t const* ix, void const* v, int32_t const* slices,
                    int64_t nslices, void const* r0, int64_t R, int64_t M, int64_t k, int32_t threads,
                    void* mu_out, double* seconds) {
        Optimized<T> oh;
        oh.h2 = csr_from<T>(n, ip, ix, v);
        oh.map.data.assign(slices, slices + nslices);
        auto ell = csr_to_ell(oh.h2);
        auto rr = static_cast<T const*>(r0);
        auto out = static_cast<T*>(mu_out);
        int64_t const nbatch = (R + k - 1) / k;
        std::atomic<int64_t> next{0};
        auto t0 = std::chrono::steady_clock::now();
        auto worker = [&] {
            Vec<T> block(n * k), mu(k * M);
            for (;;) {
                auto b = next.fetch_add(1);
                if (b >= nbatch) break;
                auto const c0 = b * k;
                auto const kk = std::min<int64_t>(k, R - c0);
                std::fill(block.begin(), block.end(), T{0});
                for (int64_t j = 0; j < kk; ++j)
                    for (int64_t i = 0; i < n; ++i) block[i * k + j] = rr[(c0 + j) * n + i];
                batch_any_width(ell, oh.map, block.data(), k, M, mu.data());
                for (int64_t j = 0; j < kk; ++j)
                    std::copy(mu.begin() + j * M, mu.begin() + (j + 1) * M, out + (c0 + j) * M);
            }
        };
        std::vector<std::thread> pool;
        for (int t = 0; t < threads; ++t) pool.emplace_back(worker);
        for (auto& t : pool) t.join();
        *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};
// The same over several independent systems at once (e.g. the flakes of a disorder
// ensemble, each with its own optimized matrix): every (system, batch) pair goes to one
// shared pool of `threads` workers, as if each system's DOS ran concurrently on one thread
// pool. Per system s: n[s] rows, CSR ip[s]/ix[s]/v[s], SliceMap slices[s] (nslices[s]),
// starters r0[s] (R x n[s]). mu_out: nsys x R x M. Returns seconds in *seconds.
template<class T> struct BenchMultiF {
    static void run(int32_t nsys, int64_t const* n, void* const* ip, void* const* ix, void* const* v,
                    void* const* slices, int64_t const* nslices, void* const* r0, int64_t R, int64_t M, int64_t k,
                    int32_t threads, void* mu_out, double* seconds) {
        std::vector<Ell<T>> ells;
        std::vector<SliceMap> maps(nsys);
        ells.reserve(nsys);
        for (int32_t s = 0; s < nsys; ++s) {
            ells.push_back(csr_to_ell(csr_from<T>(n[s], static_cast<int32_t const*>(ip[s]),
                                                  static_cast<int32_t const*>(ix[s]), v[s])));
            auto const* sl = static_cast<int32_t const*>(slices[s]);
            maps[s].data.assign(sl, sl + nslices[s]);
        }
        auto out = static_cast<T*>(mu_out);
        int64_t const nbatch = (R + k - 1) / k;
        std::atomic<int64_t> next{0};
        auto t0 = std::chrono::steady_clock::now();
        auto worker = [&] {
            Vec<T> block, mu(k * M);
            for (;;) {
                auto const item = next.fetch_add(1);
                if (item >= nbatch * nsys) break;
                auto const s = item / nbatch, b = item % nbatch;
                auto const ns = n[s];
                auto const* rr = static_cast<T const*>(r0[s]);
                auto const c0 = b * k;
                auto const kk = std::min<int64_t>(k, R - c0);
                block.assign(ns * k, T{0});
                for (int64_t j = 0; j < kk; ++j)
                    for (int64_t i = 0; i < ns; ++i) block[i * k + j] = rr[(c0 + j) * ns + i];
                batch_any_width(ells[s], maps[s], block.data(), k, M, mu.data());
                for (int64_t j = 0; j < kk; ++j)
                    std::copy(mu.begin() + j * M, mu.begin() + (j + 1) * M, out + (s * R + c0 + j) * M);
            }
        };
        std::vector<std::thread> pool;
        for (int t = 0; t < threads; ++t) pool.emplace_back(worker);
        for (auto& t : pool) t.join();
        *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};
extern "C" int orc_bench_diag_multi(int32_t dtype, int32_t nsys, int64_t const* n, void* const* ip, void* const* ix,
                                    void* const* v, void* const* slices, int64_t const* nslices, void* const* r0,
                                    int64_t R, int64_t M, int64_t k, int32_t threads, void* mu_out, double* seconds) {
    return guarded([&] {
        dispatch<BenchMultiF>(dtype, nsys, n, ip, ix, v, slices, nslices, r0, R, M, k, threads, mu_out, seconds);
    });
}

extern "C" int orc_bench_diag(int32_t dtype, int64_t n, int32_t const* ip, int32_t const* ix, void const* v, int32_t const* slices,
                   int64_t nslices, void const* r0, int64_t R, int64_t M, int64_t k, int32_t threads, void* mu_out,
                   double* seconds) {
    return guarded([&] {
        dispatch<BenchF>(dtype, n, ip, ix, v, slices, nslices, r0, R, M, k, threads, mu_out, seconds);
    });
}

