// A C++ host program that drives the GB300 KPM engine through its C ABI only
// (include/kpm_gb300.h), as pybinding's own C++ core would call a compute backend:
// kpm_config_default -> kpm_create -> kpm_scaling_factors -> kpm_moments_diag ->
// kpm_get_stats -> kpm_destroy, plus the error path of kpm_create.
//
// The fixture is a ring of N sites with hopping t, whose moments are known in closed form:
// the eigenvalues are e_k = 2 t cos(2 pi k / N) with plane-wave eigenvectors, so for a unit
// starter on any site mu_n = (1/N) sum_k T_n((e_k - b) / a), where T_n(x) = cos(n acos x),
// and mu_0 is stored halved (kpm/default/collectors.cpp:18-24). Each scalar type is checked
// against that sum: FP64 recursions to 1e-12, FP32 recursions to 1e-6.
//
// Exit status 0 when every check passes; one line per check on stdout.
#include "kpm_gb300.h"

#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

int failures = 0;

void expect(bool ok, char const* what) {
    std::printf("%s: %s\n", ok ? "ok" : "FAILED", what);
    if (!ok) ++failures;
}

template<class T>
int run_ring(int32_t scalar_type, int n, double t, int64_t num_moments, double tol) {
    std::vector<int32_t> indptr{0}, indices;
    std::vector<T> values;
    for (int i = 0; i < n; ++i) {  // sorted columns: i-1, i+1 (mod n)
        int lo = (i + n - 1) % n, hi = (i + 1) % n;
        if (lo > hi) std::swap(lo, hi);
        indices.push_back(lo);
        indices.push_back(hi);
        values.push_back(T(t));
        values.push_back(T(t));
        indptr.push_back(static_cast<int32_t>(indices.size()));
    }
    kpm_config cfg;
    kpm_config_default(&cfg);
    cfg.min_energy = -2.5;
    cfg.max_energy = 2.5;
    kpm_engine* engine = nullptr;
    if (kpm_create(scalar_type, n, indptr.data(), indices.data(), values.data(), 1, nullptr, &cfg, &engine) != KPM_OK) {
        std::printf("kpm_create failed: %s\n", kpm_last_error());
        return 1;
    }
    double a = 0, b = 0;
    if (kpm_scaling_factors(engine, 0, &a, &b) != KPM_OK) {
        std::printf("kpm_scaling_factors failed: %s\n", kpm_last_error());
        return 1;
    }
    // two starters: unit vectors on sites 0 and n/3 (the same moments by symmetry)
    std::vector<T> starters(2 * static_cast<size_t>(n), T(0));
    starters[0] = T(1);
    starters[n + n / 3] = T(1);
    int64_t m_out = 0;
    std::vector<double> out(2 * 2 * static_cast<size_t>(num_moments + 4));
    int rc = kpm_moments_diag(engine, num_moments, 2, starters.data(), 0, 0, out.data(), &m_out);
    if (rc != KPM_OK) {
        std::printf("kpm_moments_diag failed: %s\n", kpm_last_error());
        return 1;
    }
    double err = 0;
    for (int64_t m = 0; m < m_out; ++m) {
        long double ref = 0;
        for (int k = 0; k < n; ++k) {
            long double const e = 2.0L * t * std::cos(2.0L * 3.141592653589793238462643L * k / n);
            ref += std::cos(static_cast<long double>(m) * std::acos((e - b) / a));
        }
        ref /= n;
        if (m == 0) ref *= 0.5L;
        for (int v = 0; v < 2; ++v) {
            double const re = out[2 * (v * m_out + m)], im = out[2 * (v * m_out + m) + 1];
            err = std::fmax(err, std::fabs(re - static_cast<double>(ref)) + std::fabs(im));
        }
    }
    kpm_stats st{};
    kpm_get_stats(engine, &st);
    char what[160];
    std::snprintf(what, sizeof what, "ring of %d sites, type %d: %lld moments, max error %.3e (tolerance %.0e)", n,
                  scalar_type, static_cast<long long>(m_out), err, tol);
    expect(err <= tol && m_out == num_moments + ((4 - (num_moments - 2) % 4) % 4), what);
    expect(st.num_moments == m_out && st.moments_time > 0, "kpm_get_stats reports the calculation");
    expect(kpm_destroy(engine) == KPM_OK, "kpm_destroy");
    return 0;
}

}  // namespace

int main() {
    // error path: the reference's message for an inverted energy range (kpm/Core.cpp:21)
    {
        int32_t ip[] = {0, 1, 2}, ix[] = {1, 0};
        double v[] = {1.0, 1.0};
        kpm_config cfg;
        kpm_config_default(&cfg);
        cfg.min_energy = 1.0;
        cfg.max_energy = -1.0;
        kpm_engine* e = nullptr;
        int const rc = kpm_create(KPM_F64, 2, ip, ix, v, 1, nullptr, &cfg, &e);
        expect(rc == KPM_ERR_VALUE && e == nullptr &&
                   std::strcmp(kpm_last_error(), "KPM: Invalid energy range specified (min > max).") == 0,
               "kpm_create rejects min > max with the reference's message");
    }
    if (run_ring<double>(KPM_F64, 1000, -1.0, 256, 1e-12)) return 2;
    if (run_ring<std::complex<double>>(KPM_C128, 999, -1.0, 130, 1e-12)) return 2;
    if (run_ring<float>(KPM_F32, 1000, -1.0, 256, 1e-6)) return 2;
    std::printf("%s\n", failures ? "host caller: FAILED" : "host caller: all checks passed");
    return failures ? 1 : 0;
}
