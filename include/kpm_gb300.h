/*
 * kpm_gb300.h -- C ABI of the GB300 kernel polynomial method (KPM) engine.
 *
 * A drop-in compute backend for pybinding's KPM path. Every entry point takes
 * plain pointers and sizes; all arrays are HOST memory unless a parameter says
 * otherwise. Each call returns KPM_OK (0) or an error code; the message of the
 * last error on the calling thread is returned by kpm_last_error().
 *
 * The engine owns its device memory and one CUDA stream; calls on the same
 * engine must be serialised by the caller (the reference serialises them with
 * the GIL / one KPM object per thread). All device waits are bounded.
 *
 * Scalar types follow pybinding's Hamiltonian variants (float32, float64,
 * complex64, complex128; hamiltonian/Hamiltonian.hpp:48-66). Complex arrays
 * are interleaved (re, im) pairs of the real type. Hamiltonian indices are
 * int32, as in the reference (detail/config.hpp:16).
 */
#ifndef KPM_GB300_H
#define KPM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define KPM_OK 0
#define KPM_ERR_RUNTIME 1     /* std::runtime_error / logic_error -> Python RuntimeError */
#define KPM_ERR_VALUE 2       /* std::invalid_argument -> Python ValueError */
#define KPM_ERR_CUDA 3        /* a CUDA call failed */
#define KPM_ERR_TIMEOUT 4     /* a bounded device wait gave up */

/* scalar types */
#define KPM_F32 0
#define KPM_F64 1
#define KPM_C64 2
#define KPM_C128 3

/* damping kernels, kpm/Kernel.cpp:6-50 */
#define KPM_KERNEL_JACKSON 0
#define KPM_KERNEL_LORENTZ 1
#define KPM_KERNEL_DIRICHLET 2

/* recursion precision */
#define KPM_PREC_AUTO 0   /* f32 H: as KPM_PREC_FP32P; c64 H: as KPM_PREC_FP32; f64/c128 H: FP64 */
#define KPM_PREC_FP64 1   /* FP64 (f64 or c128) vectors, values and sums */
#define KPM_PREC_FP32 2   /* FP32 (f32 or c64) vectors and values, FP64 moment sums; row sums of
                             H~ x as chained FMAs */
#define KPM_PREC_FP32X 3  /* as KPM_PREC_FP32, and for real H each row sum of H~ x compensated
                             (error-free products and sums) and rounded once */
#define KPM_PREC_FP32P 4  /* as KPM_PREC_FP32, and for real H each row sum of H~ x compensated by
                             one FMA per term (Fast2Sum of the running sum and the rounded product) */

/* matrix formats accepted for API compatibility (kpm/Config.hpp:7) */
#define KPM_FORMAT_CSR 0
#define KPM_FORMAT_ELL 1

/* KPM configuration: kpm::Config (kpm/Config.hpp:23-33) plus GPU knobs. */
typedef struct kpm_config {
    double min_energy;        /* equal min/max -> bounds found by Lanczos */
    double max_energy;
    int32_t kernel;           /* KPM_KERNEL_* */
    double kernel_param;      /* lambda of the Lorentz kernel */
    int32_t matrix_format;    /* KPM_FORMAT_*; the device always uses padded ELL */
    int32_t optimal_size;     /* AlgorithmConfig::optimal_size */
    int32_t interleaved;      /* AlgorithmConfig::interleaved */
    double lanczos_precision; /* percent, default 0.002 */
    int32_t precision;        /* KPM_PREC_* */
    int32_t batch_width;      /* vectors per recursion block (upper bound); 0 = 256-byte rows */
    int32_t tile_rows;        /* rows per thread block tile; 0 = autotuned on the first call */
    int32_t fuse_steps;       /* Chebyshev steps per launch: 1, 2, or 0 = chosen by timing */
    int32_t staging;          /* diagonal step's matrix entries: 0 = chosen by timing, 1 = loaded per
                                 row, 2 = staged in shared memory a chunk of rows ahead by cp.async */
    int32_t num_threads;      /* host threads for the engine's setup work (reorder, starters, Lanczos
                                 checks); 0 = all cores. DefaultCompute's num_threads
                                 (cppmodule/src/kpm.cpp:14); the recursion itself runs on the GPU */
} kpm_config;

/* Stats of the last calculation: kpm::Stats (kpm/Stats.hpp:19-45). */
typedef struct kpm_stats {
    int64_t num_moments;
    int32_t uses_full_system;
    int64_t nnz;              /* matrix non-zeros over all steps */
    int64_t opt_nnz;
    int64_t vec;
    int64_t opt_vec;
    double multiplier;        /* vectors processed */
    int64_t matrix_memory;    /* bytes of the device matrix */
    int64_t vector_memory;    /* bytes of one KPM vector */
    double hamiltonian_time;  /* seconds: reorder + upload */
    double moments_time;      /* seconds: device time of the recursion */
    double bounds_time;       /* seconds: Lanczos */
    int32_t lanczos_loops;
    double eps;               /* opt_nnz * multiplier / moments_time */
    int32_t steps_per_launch; /* Chebyshev steps per recursion launch used last (1 or 2) */
    double gemm_time;         /* seconds: device time of the conductivity's moments GEMM (0 otherwise) */
    int32_t elems_per_lane;   /* recursion kernel lane mapping used last: vector elements per lane */
    int32_t lanes_per_row;    /*   and lanes per matrix row (their product = vectors per block) */
    int32_t staged_rows;      /*   always 0 (register loads) */
    int32_t tile_rows;        /*   rows per tile */
    int32_t unroll;           /*   rows per thread per iteration */
    double upload_time;       /* seconds (device): starter upload and scatter of the last diagonal call */
    double call_time;         /* seconds (host wall clock) of the last call, entry to return */
    int32_t gather_rows;      /* always 0 (kept for layout compatibility) */
    int32_t prefetch;         /* > 0: the diagonal step staged each warp's ELL entries in shared memory
                                 a chunk ahead (diag_pf_kernel); 3 or 4 = registers held to that many blocks per SM */
} kpm_stats;

typedef struct kpm_engine kpm_engine;

/* Message of the last failed call on this thread (empty string if none). */
const char* kpm_last_error(void);

/* Fill *cfg with the reference defaults (kpm/Config.hpp:23-33). */
void kpm_config_default(kpm_config* cfg);

/*
 * Create an engine for one Hamiltonian, or for a ragged batch of independent
 * Hamiltonians stored as one block-diagonal CSR (num_systems blocks whose first
 * rows are system_offsets[0..num_systems], system_offsets[num_systems] == rows).
 * Replaces cpb::KPM::KPM / kpm::Core::Core (cppcore/src/KPM.cpp:7-8,
 * cppcore/src/kpm/Core.cpp:17-23): copies the CSR, checks it (sorted, in
 * range, finite: hamiltonian/Hamiltonian.hpp:133-140), and raises
 * "KPM: Invalid energy range specified (min > max)." for min > max.
 */
int kpm_create(int32_t scalar_type, int64_t rows, const int32_t* indptr, const int32_t* indices,
               const void* values, int32_t num_systems, const int64_t* system_offsets,
               const kpm_config* cfg, kpm_engine** out);

/* A ragged-batch engine made of existing single-system engines (same scalar type), system i
 * being engines[i]'s Hamiltonian: their checked CSR matrices are concatenated without
 * another check, and Lanczos bounds a member has already found are kept. The members are
 * not changed and may be destroyed afterwards. The batched form of many KPM objects
 * (one per model of a parameter sweep, pybinding/parallel.py:29-70). */
int kpm_create_batch(kpm_engine* const* engines, int32_t num_engines, const kpm_config* cfg, kpm_engine** out);

/* Release the engine and its device memory. */
int kpm_destroy(kpm_engine* engine);

/* Replace the Hamiltonian (same shape rules as kpm_create). cpb::KPM::set_model
 * (cppcore/src/KPM.cpp:10-13) / Core::set_hamiltonian (Core.cpp:25-29). */
int kpm_set_hamiltonian(kpm_engine* engine, int32_t scalar_type, int64_t rows, const int32_t* indptr,
                        const int32_t* indices, const void* values, int32_t num_systems,
                        const int64_t* system_offsets);

/* Spectral bounds of one system, by FP64 Lanczos on the GPU unless set in the
 * config. kpm::Bounds (kpm/Bounds.hpp:39-72, compute/lanczos.hpp:101-154). */
int kpm_energy_bounds(kpm_engine* engine, int32_t system, double* min_energy, double* max_energy,
                      int32_t* loops);

/* KPM scaling factors a, b of one system: Bounds::scaling_factors (kpm/Bounds.hpp:57). */
int kpm_scaling_factors(kpm_engine* engine, int32_t system, double* a, double* b);

/*
 * Diagonal moments mu_n = <r|T_n(H~)|r> for caller-supplied starters: the hot
 * path (kpm/default/Compute.cpp:24-88 with kpm/calc_moments.hpp:35-89 and the
 * collectors of kpm/default/collectors.cpp:6-36), run on the GPU for every
 * system at once.
 *   starters: for each system s, num_vectors vectors of length rows_s in the
 *             ORIGINAL site order, stored [s][vector][site] in the
 *             Hamiltonian's scalar type (the one given to kpm_create; complex
 *             interleaved): exactly num_vectors * rows elements. The engine
 *             reorders them and converts them to the recursion precision.
 *   num_moments: rounded up so that (M - 2) % 4 == 0 (kpm/Kernel.hpp:9-13);
 *             the rounded count is written to *num_moments_out.
 *   out: per system [s][vector][M] moments, undamped, as complex double
 *        (2 doubles each) when `average` == 0; [s][M] averaged over the
 *        vectors (BatchAccumulator, kpm/Moments.cpp:30-48) when `average` != 0.
 *        out must hold num_systems * (average ? 1 : num_vectors) * M complex.
 *   starters_on_device: nonzero if `starters` is a device pointer (same layout).
 */
int kpm_moments_diag(kpm_engine* engine, int64_t num_moments, int64_t num_vectors, const void* starters,
                     int32_t starters_on_device, int32_t average, double* out, int64_t* num_moments_out);

/* Stochastic DOS of every system: kpm::Core::dos (cppcore/src/kpm/Core.cpp:74-90)
 * with the reference's random starters (std::mt19937 default seed per system,
 * kpm/Starter.cpp:48-84). out: [num_systems][num_energy]. */
int kpm_calc_dos(kpm_engine* engine, const double* energy, int64_t num_energy, double broadening,
                 int64_t num_random, double* out);

/* LDOS at Hamiltonian indices (system 0): kpm::Core::ldos (Core.cpp:58-72).
 * out: column-major [num_indices][num_energy]. */
int kpm_calc_ldos(kpm_engine* engine, const int64_t* indices, int64_t num_indices, const double* energy,
                  int64_t num_energy, double broadening, double* out);

/* LDOS of every system of a ragged batch at one site each (sites[s]: the local row of
 * system s), all systems in one recursion: one vector with a unit entry per system, each
 * system with its own bounds and moment count, as KPM::calc_ldos per system (KPM.cpp:55-65).
 * out is [num_systems][num_energy]. The batched form of pybinding's deferred_ldos sweeps
 * (cppmodule/src/kpm.cpp:84-91 driven by pybinding/parallel.py:29-70). */
int kpm_calc_ldos_batch(kpm_engine* engine, const int64_t* sites, const double* energy, int64_t num_energy,
                        double broadening, double* out);

/* Green's function elements (row, cols[j]) (system 0): kpm::Core::greens_vector
 * (Core.cpp:96-117). Indices are checked like cpb::KPM::calc_greens_vector
 * (KPM.cpp:110-121). out: [num_cols][num_energy] complex. */
int kpm_calc_greens(kpm_engine* engine, int64_t row, const int64_t* cols, int64_t num_cols,
                    const double* energy, int64_t num_energy, double broadening, double* out);

/* Moments <beta| op T_n(H) |alpha> (system 0): cpb::KPM::moments (KPM.cpp:19-53) +
 * kpm::Core::moments (Core.cpp:35-56). alpha/beta are complex double vectors of
 * the Hamiltonian size (beta may be NULL: beta = alpha); op is an optional
 * complex double CSR (op_rows == 0 when absent). Damped with the rounded
 * moment count; out: num_moments complex. Raises the reference's
 * "Size mismatch ..." and "The model Hamiltonian is real, but the given
 * argument '...' is complex" errors. */
int kpm_moments(kpm_engine* engine, int64_t num_moments, const double* alpha, int64_t alpha_size,
                const double* beta, int64_t beta_size, int64_t op_rows, const int32_t* op_indptr,
                const int32_t* op_indices, const double* op_values, double* out);

/* Kubo-Bastin conductivity (system 0): kpm::Core::conductivity (Core.cpp:119-150).
 * left/right: float32 site coordinates of the two directions (KPM.cpp:131-149).
 * gemm_mode: 0 = moments matrix mu_mn = sum L_m conj(R_n) in FP64 on the CUDA cores;
 *            1 = on the tensor cores (tcgen05 kind::tf32, every FP32 operand split into
 *                tf32 hi + lo, three products per pair, FP64 sums across slices): the
 *                collected vectors are stored as FP32 planes, which halves their memory
 *                for complex128; mu agrees with mode 0 to ~1e-6 relative.
 * out: num_mu complex (the caller takes the real part). */
int kpm_calc_conductivity(kpm_engine* engine, const float* left_coords, const float* right_coords,
                          const double* chemical_potential, int64_t num_mu, double broadening,
                          double temperature, int64_t num_random, int64_t num_points, int32_t gemm_mode,
                          double* out);

/* The two halves of kpm_calc_conductivity, for callers that keep or combine moments.
 * kpm_conductivity_moments: the Kubo-Bastin moments matrix of system 0 as Core::conductivity
 * builds it before damping (Core.cpp:119-145: DenseMatrixMoments of both sides,
 * MomentMultiplication::matrix_mul_add and normalize, Moments.cpp:92-126):
 * mu[m][n] = sum_r L_m conj(R_n) / num_random, row and column 0 halved; num_moments as given
 * (no rounding); out: num_moments^2 complex, column n at out + 2 n num_moments; gemm_mode
 * as for kpm_calc_conductivity.
 * kpm_kubo_bastin: reconstruct<KuboBastin> (reconstruct.hpp:90-143) of a DAMPED moments
 * matrix (multiply by g_m g_n, kpm_damping_coefficients) over num_points energy samples of
 * the engine's bounds and its scaling; out: num_mu complex. */
int kpm_conductivity_moments(kpm_engine* engine, const float* left_coords, const float* right_coords,
                             int64_t num_moments, int64_t num_random, int32_t gemm_mode, double* out);
int kpm_kubo_bastin(kpm_engine* engine, const double* moments, int64_t num_moments, const double* chemical_potential,
                    int64_t num_mu, double temperature, int64_t num_points, double* out);

/* Reverse-mode (adjoint) gradient of the averaged diagonal moments, system 0, real
 * Hamiltonians. No reference counterpart: pybinding has no gradients; the forward
 * algorithm differentiated is cpb's diagonal recursion (kpm/calc_moments.hpp:35-58,
 * kpm/default/collectors.cpp:6-36). For L = sum_n dl_dmu[n] mu_n, mu being what
 * kpm_moments_diag(engine, num_moments, num_vectors, starters, 0, average = 1, ...) returns
 * for the same starters ([num_vectors][rows], H's scalar type, site order), it writes
 * dL/dH for every stored entry of the input CSR (out_grad_values: nnz doubles, CSR order)
 * and dL/d(onsite energy) per site (out_grad_onsite: rows doubles, nullable; also where H
 * stores no diagonal). dl_dmu has round_num_moments(num_moments) entries. The scaling
 * (a, b) is held fixed. checkpoint: forward vectors are kept every `checkpoint` steps and
 * recomputed segment by segment (memory ~ (2 M / checkpoint + checkpoint) vectors);
 * >= M / 2 - 1 keeps the whole recursion (one forward pass fewer); 0 = the whole recursion
 * when it fits in half the free device memory, else ceil(sqrt(M / 2)). */
int kpm_adjoint_diag(kpm_engine* engine, int64_t num_moments, int64_t num_vectors, const void* starters,
                     const double* dl_dmu, int64_t checkpoint, double* out_grad_values, double* out_grad_onsite,
                     int64_t* num_moments_out);

/* Reverse-mode gradient of the Kubo-Bastin moments matrix (system 0; real Hamiltonians, FP64
 * recursion). No reference counterpart: pybinding has no gradients; the forward algorithm
 * differentiated is Core::conductivity's (cppcore/src/kpm/Core.cpp:119-145: DenseMatrixMoments
 * of both sides and MomentMultiplication, kpm/Moments.cpp:92-155) for caller-supplied starters
 * ([num_vectors][rows], H's scalar type, site order):
 *   mu[m][n] = (1/R) sum_r <L_m, R_n>, L_m = T_m(H~) V_l r, R_n = V_r T_n(H~) r (row/column 0 halved),
 * V = H o (x_i - x_j) from left/right coordinates. out_mu (nullable): mu, row-major [m][n], undamped.
 * With dl_dmu (row-major [m][n], nullable together with out_grad_values): the gradient of
 * L = sum_mn dl_dmu[m][n] mu[m][n] with respect to every stored entry of the input CSR
 * (out_grad_values, nnz; through the recursion and through both velocity operators) and the
 * onsite energies (out_grad_onsite, rows, nullable). The scaling (a, b) is held fixed. Keeps both
 * Chebyshev chains on the device (5 x num_moments x rows x vectors doubles). */
int kpm_adjoint_conductivity(kpm_engine* engine, const float* left_coords, const float* right_coords,
                             int64_t num_moments, int64_t num_vectors, const void* starters, const double* dl_dmu,
                             double* out_mu, double* out_grad_values, double* out_grad_onsite);

/* Stats of the last calculation (kpm/Stats.cpp:31-65; KPMStats, cppmodule/src/kpm.cpp:50-66). */
int kpm_get_stats(kpm_engine* engine, kpm_stats* out);

/* Report string: cpb::KPM::report (KPM.cpp:15-17, Stats.cpp:9-28). */
int kpm_report(kpm_engine* engine, int32_t shortform, char* buf, int64_t buf_size);

/*
 * The optimized Hamiltonian for target indices (system 0), as the test hook
 * _cpp.OptimizedHamiltonian (cppmodule/src/kpm.cpp:106-125) and
 * kpm::OptimizedHamiltonian::optimize_for (OptimizedHamiltonian.cpp:42-152):
 * scaled by 2/a, BFS-reordered from src[0] (when reorder != 0), in the
 * engine's native scalar type. Output capacities: out_indptr rows+1,
 * out_indices/out_values nnz+rows, out_map rows, out_slices rows+1,
 * out_src n_src, out_dest n_dest. Sizes come back through *out_nnz and
 * *out_num_slices; *offsets receives the SliceMap src/dest offsets.
 */
int kpm_optimized_hamiltonian(kpm_engine* engine, const int32_t* src, int64_t n_src, const int32_t* dest,
                              int64_t n_dest, int32_t reorder, int32_t* out_indptr, int32_t* out_indices,
                              void* out_values, int64_t* out_nnz, int32_t* out_map, int32_t* out_slices,
                              int64_t* out_num_slices, int32_t* out_src, int32_t* out_dest, int64_t* offsets);

/* Progress reports of the stochastic DOS (kpm_calc_dos): the progress_callback of
 * cppmodule/src/kpm.cpp:14,25,35 as kpm::DefaultCompute calls it (kpm/default/Compute.cpp:64-87,
 * 133-144): fn(-1, total) when the moments start, fn(delta, total) as parts of the recursion
 * complete (the deltas add up to total = num_random vectors), fn(total, total) at the end.
 * Called on the thread that called kpm_calc_dos, between waits on the GPU (which keeps running).
 * fn = NULL turns reporting off. */
typedef void (*kpm_progress_fn)(int64_t delta, int64_t total, void* user);
int kpm_set_progress_callback(kpm_engine* engine, kpm_progress_fn fn, void* user);

/* The engine's CUDA stream (a cudaStream_t) for interop: callers may record
 * events on it or order their own work after the engine's. No reference
 * counterpart (the reference has no device). Initialises the device. */
int kpm_get_stream(kpm_engine* engine, void** stream);

/*
 * Diagonal moments for callers that cannot allocate device memory. It has no
 * counterpart in the reference. cudaMalloc/cudaFree can synchronize the device,
 * and frameworks that own all device memory (their own pool, a fixed budget)
 * cannot accept allocations made behind their back; this call makes none.
 * The caller passes device buffers for everything: the scaled matrix H~ as
 * padded row-major ELL (col [rows][width] int32, val [rows][width][vs] of
 * vector_type, vs = 2 for KPM_F32/KPM_C64 -- each value as its FP32 high and
 * low parts -- and vs = 1 for KPM_F64/KPM_C128), the starters r0 [rows][K]
 * (K = num_vectors, interleaved per row; overwritten), a second vector buffer
 * r1 of the same size (overwritten), and out [K][num_moments] complex double.
 * num_vectors is 1 or a block of 32..512 bytes per row. The recursion's
 * scratch (tile list + per-step FP64 moment sums) is a fixed 4 MiB device
 * array inside this library, held by every GPU that loads it until the
 * process exits: calls needing more (about 16 bytes per 1024/K rows plus
 * num_moments/2 * K * 2 (real) or 3 (complex) doubles) are rejected with
 * KPM_ERR_VALUE and a message. The first call on each device looks up that
 * array's device address with the device current; make that first call
 * before any stream capture. The address is kept for the life of the process:
 * after cudaDeviceReset (or anything else that destroys the device's primary
 * context) it is stale, and this entry point must not be called again. The
 * stream must belong to the current device (checked: KPM_ERR_VALUE). Every call shares the array, so calls that
 * overlap on the GPU race; the call clears what must start at zero. Work is
 * queued on `stream` (a cudaStream_t; NULL = default stream) and the call
 * returns without waiting for it.
 */
int kpm_moments_diag_noalloc(int32_t vector_type, int64_t rows, int32_t width, const int32_t* col,
                             const void* val, int64_t num_vectors, void* r0, void* r1, int64_t num_moments,
                             double* out, void* stream);

/* Damping coefficients g_n of a kernel (kpm/Kernel.cpp:6-50). */
int kpm_damping_coefficients(int32_t kernel, double kernel_param, int64_t num_moments, double* out);

/* Moments needed for a scaled broadening, rounded (kpm/Kernel.cpp:16-20,34-37,45-48). */
int64_t kpm_required_num_moments(int32_t kernel, double kernel_param, double scaled_broadening);

#ifdef __cplusplus
}
#endif

#endif /* KPM_GB300_H */
