// Internal interface between the host engine (kpm_engine.cpp) and the CUDA
// kernels (kpm_kernels.cu). Not part of the public C ABI.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <string>

namespace kpm {

// vector / matrix element types on the device
enum VType : int { V_F32 = 0, V_F64 = 1, V_C64 = 2, V_C128 = 3 };

inline int vtype_bytes(int vt) { return vt == V_F32 ? 4 : (vt == V_C128 ? 16 : 8); }
inline bool vtype_complex(int vt) { return vt == V_C64 || vt == V_C128; }
inline bool vtype_double(int vt) { return vt == V_F64 || vt == V_C128; }
// moment sums per vector: real: (|x|^2, <y|x>), complex: (|x|^2, Re<y|x>, Im<y|x>)
inline int vtype_nv(int vt) { return vtype_complex(vt) ? 3 : 2; }
// matrix values per ELL entry: FP32 types store (hi, lo) pairs of an FP64 value
inline int vtype_vs(int vt) { return vtype_double(vt) ? 1 : 2; }

// A tile: rows [row_begin, row_end) of one system for one batch of vectors.
struct Tile {
    int32_t row_begin, row_end, system, batch;
};

// One step of the diagonal recursion, y <- H~ x - y (or y <- H~ x / 2 when init),
// with the moment sums m2 += |x_r|^2, m3 += conj(y_r) x_r per vector accumulated
// into acc[((system * nbatch + batch) * K + v) * NV + q].
struct DiagStep {
    int vtype;
    int E, LPR;               // K = E * LPR vectors per batch
    const int32_t* col;       // [rows_total][W]
    const void* val;          // [rows_total][W][vs], vtype (vs = vtype_vs)
    int W;
    const void* x;            // [nbatch][rows_total][K]
    void* y;
    int64_t batch_stride;     // rows_total * K elements
    const Tile* tiles;
    int num_tiles;
    int32_t row_limit;        // rows >= row_limit are skipped (optimal size)
    int nbatch;
    double* acc;
    bool init;
    int unroll = 1;           // rows per thread per iteration (1 or 2), chosen by the autotuner
    int prefetch = 0;         // > 0: ELL entries copied to shared memory a chunk ahead (diag_pf_kernel),
                              // register allocation for 3 or 4 resident blocks per SM (3 or 4);
                              // chosen by the autotuner; unroll is then 1
    int compensated = 0;      // FP32 real vectors, row sums of H~ x: 0 chained FMAs, 1 compensated by
                              // one FMA per term (Fast2Sum), 2 compensated by exact products and
                              // TwoSum (rounded once; one row per thread)
    bool real_matrix = false; // complex vectors with real H~ values: val holds [rows][W][vs] of the
                              // real type (vs of that type: hi/lo pairs for FP32)
};

// Off-diagonal step: y <- H~ x - y (or H~ x / 2 when init), optional fused dot
// acc[batch*K+v] += <gamma_r | y_r> (complex sums, 2 doubles) when gamma != nullptr,
// optional store of y into `store` (dense matrix of vectors, row n).
struct OffStep {
    int vtype;
    int E, LPR;
    const int32_t* col;
    const void* val;
    int W;
    const void* x;
    void* y;
    int64_t batch_stride;
    const Tile* tiles;
    int num_tiles;
    int32_t row_limit;
    bool init;
    const void* gamma;        // [rows_total] (single vector), nullable
    double* acc;
};

// Dense-collection step for the Kubo-Bastin moments (kpm/default/collectors.cpp:78-107):
// y <- H~ x - y (or H~ x / 2 when init) and, per row, optionally
//   zx[r] = x[r]                       (store T_{n-1}: the left vectors)
//   zv[r] = sum_j val2[r][j] x[c_j]    (store V T_{n-1}: the right vectors)
struct DenseStep {
    int vtype;
    int E, LPR;
    const int32_t* col;
    const void* val;
    const void* val2;         // nullable
    int W;
    const void* x;
    void* y;
    void* zx;                 // nullable, [rows][K]
    void* zv;                 // nullable, [rows][K]
    float* zre;               // nullable: FP32 planes [rows][K] of the collected vector (V r when
    float* zim;               // val2 is set, else r); zim for complex types only
    const Tile* tiles;
    int num_tiles;
    bool init;
};

// Adjoint of the diagonal recursion (real types): one launch of
//   out = S x - yprev (or S x / 2 when half) + a0 v0 + am vm + ap vp
// plus, when gt is set, gt[r][j] += sum_k x[col[r][j]][k] * g[r][k] ([rows][W]) and
// gd[r] += sum_k x[r][k] * g[r][k] ([rows]), both in the vector type's precision.
struct AdjStep {
    int vtype;
    int E, LPR;
    const int32_t* col;
    const void* val;
    int W;
    const void* x;
    const void* yprev;        // nullable; may alias out
    void* out;                // nullable (gradient only)
    bool half;
    const void* v0;           // nullable
    const void* vm;           // nullable
    const void* vp;           // nullable
    double a0, am, ap;
    const void* g;            // row vectors of the gradient term (with gt)
    void* gt;                 // nullable; gradient sums [rows][W]: FP64 for FP64 vectors, (hi, lo) FP32 pairs
                              // (float2) for FP32 ones
    void* gd;                 // set with gt; [rows], the same type
    const Tile* tiles;
    int num_tiles;
};

// Two recursion steps in one launch (steps n and n+1; P = T_{n-2} -> T_n, Q = T_{n-1} -> T_{n+1}).
// items: [2 * num_tiles] work items (tile * 2 + phase) in dependency order; band: [num_tiles][2]
// tile range whose phase A must finish before phase B of the tile; flags: [num_tiles] sequence
// number of the last finished phase A (persist across launches; seq grows per launch);
// counter: item dispenser of this launch, zeroed beforehand.
struct DiagPair {
    int vtype;
    int E, LPR;
    const int32_t* col;
    const void* val;
    int W;
    void* P;
    void* Q;
    int64_t batch_stride;
    const Tile* tiles;
    const int32_t* items;
    const int32_t* band;
    int num_tiles;
    int nbatch;
    int* flags;
    int seq;
    unsigned* counter;
    double* accA;
    double* accB;
    int* error;
    int spin_limit;
};

cudaError_t launch_diag_step(DiagStep const& a, cudaStream_t s);
cudaError_t launch_diag_pair(DiagPair const& a, cudaStream_t s);
cudaError_t launch_dense_step(DenseStep const& a, cudaStream_t s);

// mu[n * M + m] += sum_i A[m * I + i] * conj(B[n * I + i]) in FP64 (complex double mu),
// A and B in vtype; split over I with FP64 atomics.
cudaError_t launch_mu_gemm_fp64(int vtype, void const* A, void const* B, int64_t M, int64_t I, double* mu,
                                cudaStream_t s);

// mu += L R^H on tensor cores (tcgen05 kind::tf32, three-product hi/lo split; FP64 atomics).
// Operands are FP32 planes [M][ld] (row m = vector L_m / R_m over I = rows x vectors
// elements, 16-byte aligned, ld * 4 a multiple of 16); cplx adds the imaginary planes.
// mu is complex double [n * M + m]. err is set when a bounded device wait gives up.
cudaError_t launch_mu_gemm_tc(bool cplx, float const* a_re, float const* a_im, float const* b_re, float const* b_im,
                              int64_t M, int64_t I, int64_t ld, int group_kb, double* mu, int* err, cudaStream_t s);

// Kubo-Bastin (kpm/reconstruct.hpp:90-143) in FP64:
// sum_nm[e] = 1/(1-en^2)^2 * sum_{m,n} mu(m,n) (A_n T_m + conj(A_m) T_n), en = scaled sample e
cudaError_t launch_kubo_sum(double const* mu, int64_t M, double const* scaled_samples, int ns, double* sum_nm,
                            cudaStream_t s);
// out[j] = prefix * coeff * sum_e w_e fd(en_e, mu_j) sum_nm[e]
cudaError_t launch_kubo_integrate(double const* sum_nm, double const* scaled_samples, int ns,
                                  double const* scaled_mu, int nmu, double inv_kbt, double coeff, double prefix,
                                  double* out, cudaStream_t s);
cudaError_t launch_off_step(OffStep const& a, cudaStream_t s);
cudaError_t launch_adj_step(AdjStep const& a, cudaStream_t s);
// out = a x + b y over n elements of a real vector type (y nullable)
// dst[0..bytes) = src[0..bytes), both 16-byte aligned; src may be host memory that the GPU
// reads through the host page tables (a copy at the link's rate, no staging)
cudaError_t launch_copy(void* dst, void const* src, size_t bytes, cudaStream_t s);
// Y[m][i] = sum_n C[m][n] X[n][i] in FP64 (C: M x M row-major; X, Y: M rows of I doubles)
cudaError_t launch_dense_combine(double const* C, double const* X, double* Y, int M, int64_t I, cudaStream_t s);
cudaError_t launch_axpby(int vtype, int64_t n, double a, void const* x, double b, void const* y, void* out,
                         cudaStream_t s);
bool diag_shape_supported(int vtype, int E, int LPR);
// diag_step_kernel instantiations, thinner lane mappings included (what launch_diag_step runs)
bool diag_step_supported(int vtype, int E, int LPR);
// the prefetched-entries step (DiagStep::prefetch) fits rows of W entries in shared memory
bool diag_pf_supported(int vtype, int W, int LPR);

// moments from the accumulated sums: out[(s*nbatch*K + v) * M + n] complex double,
// or averaged over `nvec` vectors per system into out[s * M + n] when average.
cudaError_t launch_collect_diag(int vtype, double const* acc, int num_systems, int nbatch, int K,
                                int64_t half_M, int64_t M, int64_t nvec, bool average, double* out,
                                cudaStream_t s);

cudaError_t launch_average(double const* per_vec, int num_systems, int64_t nvec, int64_t M, double* out,
                           cudaStream_t s);

// unit starters: dst[(b * rows_total + pos[v]) * K + j] = 1 for v = b*K + j < nvec
cudaError_t launch_set_units(int vtype, void* dst, int32_t const* pos, int64_t nvec, int K, int64_t rows_total,
                             cudaStream_t s);

// scatter host-order starters (scalar type `stype`, same codes as VType) into the
// reordered, batched device layout of type `vtype`:
// dst[(b * rows_total + map[g]) * K + j] = src[(s, v, i)], v = b*K + j
cudaError_t launch_scatter_starters(int stype, int vtype, void const* src, void* dst, int32_t const* map,
                                    int64_t const* sys_offsets, int num_systems, int64_t nvec,
                                    int K, int nbatch, int64_t rows_total, cudaStream_t s);

// gather y[dest[i]] (batch 0, vector 0) into out[n * ndest + i] as complex double
cudaError_t launch_gather_rows(int vtype, void const* y, int32_t const* dest, int ndest, double* out,
                               cudaStream_t s);

// Lanczos (FP64 or complex FP64, all systems in lockstep, CSR per system in global rows)
// A: t = H v1; v0 = t - sqrt(nrm_prev[s]) v0; alpha[s] = sum Re(conj(t) v1)
// B: v0 -= alpha[s] v1; nrm[s] = sum |v0|^2
// C: v0 *= 1/sqrt(nrm[s])
// The sums of A and B go through per-tile partials (`part`, num_tiles doubles) reduced per
// system in a fixed order (tiles sys_tiles[s] .. sys_tiles[s + 1] - 1): bit-reproducible.
cudaError_t launch_lanczos_a(bool cplx, int32_t const* ip, int32_t const* ix, void const* v,
                             void const* v1, void* v0, Tile const* tiles, int num_tiles,
                             double const* nrm_prev, double* part, int32_t const* sys_tiles, int nsys,
                             double* alpha, cudaStream_t s);
cudaError_t launch_lanczos_b(bool cplx, void const* v1, void* v0, Tile const* tiles, int num_tiles,
                             double const* alpha, double* part, int32_t const* sys_tiles, int nsys, double* nrm,
                             cudaStream_t s);
cudaError_t launch_lanczos_c(bool cplx, void* v0, Tile const* tiles, int num_tiles, double const* nrm,
                             cudaStream_t s);

// reconstruction in FP64: out[c * ne + e] = k/sqrt(1-E^2) sum_n Re(mu[c*M+n]) cos(n acos E)
cudaError_t launch_spectral_density(double const* mu, int64_t M, int cols, double const* energy, int ne,
                                    double a, double b, double* out, cudaStream_t s);
// Green's: out[c * ne + e] = -2i/(a sqrt(1-E^2)) sum_n mu[c*M+n] exp(-i n acos E) (complex)
cudaError_t launch_greens(double const* mu, int64_t M, int cols, double const* energy, int ne, double a,
                          double b, double* out, cudaStream_t s);

// Record the message that kpm_last_error() returns on this thread.
void set_last_error(std::string const& msg);

}  // namespace kpm
