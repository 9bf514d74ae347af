/*
 * kpm_lattice.h -- C ABI of the GPU builder of KPM inputs: tight-binding Hamiltonians
 * in pybinding's site order, built on the device and returned as host CSR arrays.
 *
 * Replaces, for the two lattices the KPM workloads use, pybinding's host model build:
 *   - foundation positions       cppcore/src/system/Foundation.cpp:25-48 (generate_positions)
 *   - polygon membership         cppcore/src/system/Shape.cpp:54-88 (Polygon::contains)
 *   - dangling-site removal      cppcore/src/system/Foundation.cpp:50-101 (the k-core of the site graph)
 *   - final site indices         cppcore/src/system/Foundation.cpp:127-164 (valid sites, sublattice-major)
 *   - Hamiltonian CSR            cppcore/include/hamiltonian/Hamiltonian.hpp:74-100 (build_main:
 *                                hoppings inserted for the owning site and mirrored as conjugates,
 *                                zero onsite energies not stored, sorted columns per row)
 *
 * The results are identical, bit for bit, to the host build: positions in float32 with the
 * reference's operation order, integer structure exact, values copied or conjugated.
 * Modifiers stay with the caller: kpm_lattice_sites / kpm_lattice_hoppings return the
 * positions and the hopping list (in the host build's order) for the caller to evaluate
 * onsite and hopping energies, which kpm_lattice_csr then assembles.
 *
 * Status codes and kpm_last_error() are those of kpm_gb300.h. All arrays are HOST memory.
 */
#ifndef KPM_LATTICE_H
#define KPM_LATTICE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct kpm_lattice kpm_lattice; /* device-side build state of one lattice */

/* A two-sublattice lattice with three hoppings per A site (graphene), in 2D. Sites are
 * generated sublattice-major, then along a2, then along a1 (fastest), on a foundation of
 * s0 x s1 cells whose cell (0, 0) sits at `origin`. Every float is the float32 value the
 * host build uses. */
typedef struct kpm_honeycomb {
    int32_t s0, s1;          /* foundation cells along a1 and a2 */
    float origin[3];         /* position of cell (0, 0) */
    float a1[3], a2[3];      /* lattice vectors */
    float sub[2][3];         /* sublattice offsets: A, B */
    int32_t hop[3][2];       /* cell offsets (along a1, a2) from an A site to its three B neighbours */
    int32_t min_neighbors;   /* sites with fewer valid neighbours are removed (repeatedly) */
} kpm_honeycomb;

/* Build the sites of a honeycomb foundation cut by a polygon (num_vertices (x, y) pairs,
 * float32; Shape.cpp:54-88) and remove dangling sites. */
int kpm_lattice_honeycomb(const kpm_honeycomb* params, const float* vertices, int32_t num_vertices,
                          kpm_lattice** out);

/* Periodic simple cubic L^3 lattice (L >= 3), site index (z L + y) L + x, six hoppings per site. */
int kpm_lattice_cubic(int32_t L, kpm_lattice** out);

/* Number of sites, of sites in the first sublattice, of hoppings (each bond once), and the
 * largest possible number of CSR entries (bonds twice plus one diagonal per site). */
int kpm_lattice_sizes(const kpm_lattice* h, int64_t* num_sites, int64_t* num_sub0, int64_t* num_hoppings,
                      int64_t* max_nnz);

/* Site positions (float32, num_sites each). */
int kpm_lattice_sites(kpm_lattice* h, float* x, float* y, float* z);

/* The hopping list in the host build's order: for each of the three directions, the A
 * sites (ascending) whose neighbour exists; rows are A sites, cols their B neighbours.
 * For the cubic lattice, whose entries are all listed (no mirroring): for each of the six
 * directions (+x, -x, +y, -y, +z, -z), every site; num_hoppings is then 6 L^3. */
int kpm_lattice_hoppings(kpm_lattice* h, int32_t* rows, int32_t* cols);

/* Assemble the Hamiltonian CSR (dtype KPM_F32 / F64 / C64 / C128 of kpm_gb300.h; complex
 * values are (re, im) pairs). `hopping` is one value of dtype used for every bond, or
 * NULL when `hopping_values` (num_hoppings values in kpm_lattice_hoppings order) is given;
 * a bond's mirrored entry holds the conjugate (the cubic lattice takes a single value).
 * `onsite` (num_sites values) may be NULL;
 * zero onsite energies are not stored. indptr has num_sites + 1 entries; indices and
 * values room for `capacity` entries; the entry count is written to *nnz. */
int kpm_lattice_csr(kpm_lattice* h, int32_t dtype, const void* hopping, const void* hopping_values,
                    const void* onsite, int32_t* indptr, int32_t* indices, void* values, int64_t capacity,
                    int64_t* nnz);

/* Device time of the last kpm_lattice_honeycomb / kpm_lattice_cubic and kpm_lattice_csr calls,
 * seconds, and the number of kernels this builder has launched. */
int kpm_lattice_times(const kpm_lattice* h, double* build_time, double* csr_time, int64_t* launches);

int kpm_lattice_destroy(kpm_lattice* h);

#ifdef __cplusplus
}
#endif

#endif /* KPM_LATTICE_H */
