// _kpm_gb300: the pybind11 module over the engine's C ABI (include/kpm_gb300.h).
//
// The Python-facing half of the boundary, in the place of pybinding's own pybind11 KPM
// module (cppmodule/src/kpm.cpp:8-102): an Engine class per Hamiltonian (or ragged batch of
// Hamiltonians) whose methods are the KPM calculations, NumPy arrays in and out, errors
// raised with the reference's exception types (std::invalid_argument -> ValueError, every
// other failure -> RuntimeError, as pybind11 translates them for the reference) and the GIL
// released while the GPU works (cppmodule/src/kpm.cpp:78-83 releases it for calc_*).
// Nothing here computes: every call goes through a kpm_* function of libkpm_gb300.so.
#include <pybind11/functional.h>
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <complex>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "kpm_gb300.h"

namespace py = pybind11;

namespace {

void check(int rc) {
    if (rc == KPM_OK) return;
    std::string const msg = kpm_last_error();
    if (rc == KPM_ERR_VALUE) throw py::value_error(msg);
    throw std::runtime_error(msg);
}

template<class T>
using carr = py::array_t<T, py::array::c_style | py::array::forcecast>;

int kernel_code(std::string const& name) {
    if (name == "jackson") return KPM_KERNEL_JACKSON;
    if (name == "lorentz") return KPM_KERNEL_LORENTZ;
    if (name == "dirichlet") return KPM_KERNEL_DIRICHLET;
    throw py::value_error("unknown kernel '" + name + "'");
}

// kpm_config from keyword arguments (the names of pybinding_gb300._native.make_config)
kpm_config make_config(py::dict kw) {
    kpm_config c;
    kpm_config_default(&c);
    for (auto item : kw) {
        auto const key = item.first.cast<std::string>();
        py::handle v = item.second;
        if (key == "energy_range") {
            auto const r = v.cast<std::pair<double, double>>();
            c.min_energy = r.first;
            c.max_energy = r.second;
        } else if (key == "kernel") {
            c.kernel = kernel_code(v.cast<std::string>());
        } else if (key == "kernel_param") {
            c.kernel_param = v.cast<double>();
        } else if (key == "matrix_format") {
            c.matrix_format = v.cast<std::string>() == "ELL" ? KPM_FORMAT_ELL : KPM_FORMAT_CSR;
        } else if (key == "optimal_size") {
            c.optimal_size = v.cast<bool>();
        } else if (key == "interleaved") {
            c.interleaved = v.cast<bool>();
        } else if (key == "lanczos_precision") {
            c.lanczos_precision = v.cast<double>();
        } else if (key == "precision") {
            auto const p = v.cast<std::string>();
            if (p == "auto") c.precision = KPM_PREC_AUTO;
            else if (p == "fp64") c.precision = KPM_PREC_FP64;
            else if (p == "fp32") c.precision = KPM_PREC_FP32;
            else if (p == "fp32x") c.precision = KPM_PREC_FP32X;
            else if (p == "fp32p") c.precision = KPM_PREC_FP32P;
            else throw py::value_error("precision must be 'auto', 'fp64', 'fp32', 'fp32p' or 'fp32x'");
        } else if (key == "batch_width") {
            c.batch_width = v.cast<int32_t>();
        } else if (key == "tile_rows") {
            c.tile_rows = v.cast<int32_t>();
        } else if (key == "fuse_steps") {
            c.fuse_steps = v.cast<int32_t>();
        } else if (key == "staging") {
            auto const st = v.cast<std::string>();
            if (st == "auto") c.staging = 0;
            else if (st == "registers") c.staging = 1;
            else if (st == "prefetch") c.staging = 2;
            else throw py::value_error("staging must be 'auto', 'registers' or 'prefetch'");
        } else if (key == "num_threads") {
            c.num_threads = (v.is_none() || py::isinstance<py::str>(v)) ? 0 : v.cast<int32_t>();
        } else {
            throw py::type_error("unknown KPM configuration key '" + key + "'");
        }
    }
    return c;
}

// A SciPy CSR matrix (anything scipy.sparse.csr_matrix accepts) with sorted indices.
struct Csr {
    int64_t rows = 0;
    int32_t stype = KPM_F32;
    carr<int32_t> indptr, indices;
    py::array values;
    py::dtype dtype;
};

Csr csr_of(py::object h) {
    auto sp = py::module_::import("scipy.sparse");
    py::object m = sp.attr("csr_matrix")(h);
    if (!m.attr("has_sorted_indices").cast<bool>()) {
        m = m.attr("copy")();
        m.attr("sort_indices")();
    }
    Csr c;
    auto const shape = m.attr("shape").cast<std::pair<int64_t, int64_t>>();
    c.rows = shape.first;
    c.indptr = carr<int32_t>(m.attr("indptr"));
    c.indices = carr<int32_t>(m.attr("indices"));
    py::array data = m.attr("data");
    c.dtype = data.dtype();
    auto np = py::module_::import("numpy");
    char const kind = c.dtype.kind();
    auto const size = c.dtype.itemsize();
    if (kind == 'f' && size == 4) c.stype = KPM_F32;
    else if (kind == 'f' && size == 8) c.stype = KPM_F64;
    else if (kind == 'c' && size == 8) c.stype = KPM_C64;
    else if (kind == 'c' && size == 16) c.stype = KPM_C128;
    else throw py::type_error("unsupported Hamiltonian dtype " + py::str(c.dtype).cast<std::string>());
    c.values = np.attr("ascontiguousarray")(data);
    return c;
}

int64_t round_num_moments(int64_t n) {  // kpm/Kernel.hpp:9-13
    if (n < 2) return 2;
    return n + ((4 - (n - 2) % 4) % 4);
}

void progress_trampoline(int64_t delta, int64_t total, void* user) {
    py::gil_scoped_acquire gil;
    auto* fn = static_cast<py::object*>(user);
    try {
        (*fn)(delta, total);
    } catch (py::error_already_set& e) {  // a failing callback must not unwind through the engine
        e.discard_as_unraisable("kpm progress callback");
    }
}

class Engine {
public:
    Engine(py::object hamiltonian, py::dict config, py::object system_offsets) : cfg_(make_config(config)) {
        Csr c = csr_of(hamiltonian);
        set_shape(c, system_offsets);
        kpm_engine* h = nullptr;
        check(kpm_create(c.stype, c.rows, c.indptr.data(), c.indices.data(), c.values.data(), nsys_,
                         offsets_ptr(), &cfg_, &h));
        h_ = h;
    }
    // a ragged batch made of existing engines (kpm_create_batch)
    Engine(std::vector<Engine*> const& members, py::dict config) : cfg_(make_config(config)) {
        if (members.empty()) throw py::value_error("no engines to batch");
        std::vector<kpm_engine*> hs;
        std::vector<int64_t> off{0};
        for (auto* m : members) {
            hs.push_back(m->handle());
            off.push_back(off.back() + m->rows_);
            nnz_ += m->nnz_;
        }
        rows_ = off.back();
        nsys_ = static_cast<int32_t>(members.size());
        dtype_ = members.front()->dtype_;
        offsets_ = carr<int64_t>(static_cast<py::ssize_t>(off.size()));
        std::copy(off.begin(), off.end(), offsets_.mutable_data());
        kpm_engine* h = nullptr;
        check(kpm_create_batch(hs.data(), nsys_, &cfg_, &h));
        h_ = h;
    }
    ~Engine() { close(); }
    Engine(Engine const&) = delete;
    Engine& operator=(Engine const&) = delete;

    void close() {
        if (h_) kpm_destroy(h_);
        h_ = nullptr;
    }
    kpm_engine* handle() const {
        if (!h_) throw std::runtime_error("the engine is closed");
        return h_;
    }

    void set_hamiltonian(py::object hamiltonian, py::object system_offsets) {
        Csr c = csr_of(hamiltonian);
        set_shape(c, system_offsets);
        check(kpm_set_hamiltonian(handle(), c.stype, c.rows, c.indptr.data(), c.indices.data(), c.values.data(),
                                  nsys_, offsets_ptr()));
    }

    py::tuple energy_bounds(int32_t system) {
        double mn = 0, mx = 0;
        int32_t loops = 0;
        {
            py::gil_scoped_release nogil;
            check(kpm_energy_bounds(handle(), system, &mn, &mx, &loops));
        }
        return py::make_tuple(mn, mx, loops);
    }

    py::tuple scaling_factors(int32_t system) {
        double a = 0, b = 0;
        {
            py::gil_scoped_release nogil;
            check(kpm_scaling_factors(handle(), system, &a, &b));
        }
        return py::make_tuple(a, b);
    }

    // starters [system][vector][site] in the Hamiltonian's dtype (host), or a device address
    py::array moments_diag(int64_t num_moments, py::object starters, bool average, py::object on_device_ptr,
                           py::object num_vectors) {
        int64_t const M = round_num_moments(num_moments);
        int64_t nvec = 0;
        void const* src = nullptr;
        int32_t dev = 0;
        py::array keep;
        if (!on_device_ptr.is_none()) {
            if (num_vectors.is_none() || num_vectors.cast<int64_t>() < 1)
                throw py::value_error("num_vectors is required with a device pointer");
            nvec = num_vectors.cast<int64_t>();
            src = reinterpret_cast<void const*>(on_device_ptr.cast<uintptr_t>());
            dev = 1;
        } else {
            keep = contiguous(starters);
            if (keep.size() == 0 || keep.size() % rows_)
                throw py::value_error("starters must hold num_vectors * " + std::to_string(rows_) + " elements");
            nvec = keep.size() / rows_;
            src = keep.data();
        }
        int64_t const cols = average ? nsys_ : nsys_ * nvec;
        auto out = carr<std::complex<double>>({cols, M});
        int64_t nout = 0;
        {
            py::gil_scoped_release nogil;
            check(kpm_moments_diag(handle(), num_moments, nvec, src, dev, average ? 1 : 0,
                                   reinterpret_cast<double*>(out.mutable_data()), &nout));
        }
        if (average) return out.reshape({static_cast<int64_t>(nsys_), M});
        return out.reshape({static_cast<int64_t>(nsys_), nvec, M});
    }

    py::array calc_dos(carr<double> energy, double broadening, int64_t num_random) {
        auto out = carr<double>({static_cast<py::ssize_t>(nsys_), energy.size()});
        py::gil_scoped_release nogil;
        check(kpm_calc_dos(handle(), energy.data(), energy.size(), broadening, num_random, out.mutable_data()));
        return out;
    }

    py::array calc_ldos(carr<int64_t> indices, carr<double> energy, double broadening) {
        auto out = carr<double>({indices.size(), energy.size()});
        {
            py::gil_scoped_release nogil;
            check(kpm_calc_ldos(handle(), indices.data(), indices.size(), energy.data(), energy.size(), broadening,
                                out.mutable_data()));
        }
        return py::array(out.attr("T"));  // (energy, indices)
    }

    py::array calc_ldos_batch(carr<int64_t> sites, carr<double> energy, double broadening) {
        if (sites.size() != nsys_)
            throw py::value_error("one LDOS site per system (" + std::to_string(nsys_) + ")");
        auto out = carr<double>({static_cast<py::ssize_t>(nsys_), energy.size()});
        py::gil_scoped_release nogil;
        check(kpm_calc_ldos_batch(handle(), sites.data(), energy.data(), energy.size(), broadening,
                                  out.mutable_data()));
        return out;
    }

    py::array calc_greens(int64_t row, carr<int64_t> cols, carr<double> energy, double broadening) {
        auto out = carr<std::complex<double>>({cols.size(), energy.size()});
        py::gil_scoped_release nogil;
        check(kpm_calc_greens(handle(), row, cols.data(), cols.size(), energy.data(), energy.size(), broadening,
                              reinterpret_cast<double*>(out.mutable_data())));
        return out;
    }

    // <beta| op T_n(H) |alpha> (KPM::moments, KPM.cpp:19-53); beta/op may be None or empty
    py::array moments(int64_t num_moments, carr<std::complex<double>> alpha, py::object beta, py::object op) {
        carr<std::complex<double>> b;
        bool have_beta = !beta.is_none() && py::len(beta) > 0;
        if (have_beta) b = carr<std::complex<double>>(py::module_::import("numpy").attr("ravel")(beta));
        int64_t orows = 0;
        carr<int32_t> oip, oix;
        carr<std::complex<double>> ov;
        if (!op.is_none() && op.attr("shape").cast<std::pair<int64_t, int64_t>>().first != 0) {
            auto sp = py::module_::import("scipy.sparse");
            py::object o = sp.attr("csr_matrix")(op).attr("astype")(py::dtype::of<std::complex<double>>());
            auto const shape = o.attr("shape").cast<std::pair<int64_t, int64_t>>();
            orows = shape.first == shape.second ? shape.first : -1;
            oip = carr<int32_t>(o.attr("indptr"));
            oix = carr<int32_t>(o.attr("indices"));
            ov = carr<std::complex<double>>(o.attr("data"));
        }
        auto out = carr<std::complex<double>>(static_cast<py::ssize_t>(num_moments));
        check(kpm_moments(handle(), num_moments, reinterpret_cast<double const*>(alpha.data()), alpha.size(),
                          have_beta ? reinterpret_cast<double const*>(b.data()) : nullptr,
                          have_beta ? b.size() : 0, orows, orows ? oip.data() : nullptr,
                          orows ? oix.data() : nullptr,
                          orows ? reinterpret_cast<double const*>(ov.data()) : nullptr,
                          reinterpret_cast<double*>(out.mutable_data())));
        return out;
    }

    py::array calc_conductivity(carr<float> left, carr<float> right, carr<double> chemical_potential,
                                double broadening, double temperature, int64_t num_random, int64_t num_points,
                                int32_t gemm_mode) {
        auto out = carr<std::complex<double>>(chemical_potential.size());
        py::gil_scoped_release nogil;
        check(kpm_calc_conductivity(handle(), left.data(), right.data(), chemical_potential.data(),
                                    chemical_potential.size(), broadening, temperature, num_random, num_points,
                                    gemm_mode, reinterpret_cast<double*>(out.mutable_data())));
        return out;
    }

    // gradient of L = sum_n dl_dmu[n] mu_n with respect to the stored entries and onsite energies
    py::tuple adjoint_diag(int64_t num_moments, py::object starters, carr<double> dl_dmu, int64_t checkpoint) {
        int64_t const M = round_num_moments(num_moments);
        if (dl_dmu.size() != M)
            throw py::value_error("dl_dmu must hold round_num_moments(num_moments) = " + std::to_string(M) +
                                  " entries");
        py::array keep = contiguous(starters);
        if (keep.size() == 0 || keep.size() % rows_)
            throw py::value_error("starters must hold num_vectors * " + std::to_string(rows_) + " elements");
        int64_t const nvec = keep.size() / rows_;
        auto gv = carr<double>(static_cast<py::ssize_t>(nnz_));
        auto go = carr<double>(static_cast<py::ssize_t>(rows_));
        int64_t nout = 0;
        {
            py::gil_scoped_release nogil;
            check(kpm_adjoint_diag(handle(), num_moments, nvec, keep.data(), dl_dmu.data(), checkpoint,
                                   gv.mutable_data(), go.mutable_data(), &nout));
        }
        return py::make_tuple(gv, go);
    }

    // Kubo-Bastin moments matrix of explicit starters and, with dl_dmu, its gradient
    py::tuple adjoint_conductivity(carr<float> left, carr<float> right, int64_t num_moments, py::object starters,
                                   py::object dl_dmu) {
        py::array keep = contiguous(starters);
        if (keep.size() == 0 || keep.size() % rows_)
            throw py::value_error("starters must hold num_vectors * " + std::to_string(rows_) + " elements");
        int64_t const M = num_moments;
        auto mu = carr<double>({M, M});
        carr<double> w;
        py::object gv = py::none(), go = py::none();
        double* gvp = nullptr;
        double* gop = nullptr;
        if (!dl_dmu.is_none()) {
            w = carr<double>(dl_dmu);
            if (w.ndim() != 2 || w.shape(0) != M || w.shape(1) != M)
                throw py::value_error("dl_dmu must have shape (num_moments, num_moments)");
            auto a = carr<double>(static_cast<py::ssize_t>(nnz_));
            auto b = carr<double>(static_cast<py::ssize_t>(rows_));
            gvp = a.mutable_data();
            gop = b.mutable_data();
            gv = a;
            go = b;
        }
        {
            py::gil_scoped_release nogil;
            check(kpm_adjoint_conductivity(handle(), left.data(), right.data(), M, keep.size() / rows_, keep.data(),
                                           gvp ? w.data() : nullptr, mu.mutable_data(), gvp, gop));
        }
        return py::make_tuple(mu, gv, go);
    }

    void set_progress_callback(py::object fn) {
        progress_ = fn;
        if (fn.is_none()) check(kpm_set_progress_callback(handle(), nullptr, nullptr));
        else check(kpm_set_progress_callback(handle(), &progress_trampoline, &progress_));
    }

    py::object stats() {  // attribute access, like pybinding's KPMStats
        kpm_stats s{};
        check(kpm_get_stats(handle(), &s));
        py::dict d;
        d["num_moments"] = s.num_moments;
        d["uses_full_system"] = s.uses_full_system != 0;
        d["nnz"] = s.nnz;
        d["opt_nnz"] = s.opt_nnz;
        d["vec"] = s.vec;
        d["opt_vec"] = s.opt_vec;
        d["multiplier"] = s.multiplier;
        d["matrix_memory"] = s.matrix_memory;
        d["vector_memory"] = s.vector_memory;
        d["hamiltonian_time"] = s.hamiltonian_time;
        d["moments_time"] = s.moments_time;
        d["bounds_time"] = s.bounds_time;
        d["lanczos_loops"] = s.lanczos_loops;
        d["eps"] = s.eps;
        d["steps_per_launch"] = s.steps_per_launch;
        d["gemm_time"] = s.gemm_time;
        d["elems_per_lane"] = s.elems_per_lane;
        d["lanes_per_row"] = s.lanes_per_row;
        d["tile_rows"] = s.tile_rows;
        d["unroll"] = s.unroll;
        d["prefetch"] = s.prefetch;
        d["upload_time"] = s.upload_time;
        d["call_time"] = s.call_time;
        return py::module_::import("types").attr("SimpleNamespace")(**d);
    }

    std::string report(bool shortform) {
        std::string buf(4096, '\0');
        check(kpm_report(handle(), shortform ? 1 : 0, &buf[0], static_cast<int64_t>(buf.size())));
        buf.resize(std::char_traits<char>::length(buf.c_str()));
        return buf;
    }

    uintptr_t stream() {
        void* p = nullptr;
        check(kpm_get_stream(handle(), &p));
        return reinterpret_cast<uintptr_t>(p);
    }

    int64_t rows_ = 0;
    int32_t nsys_ = 1;
    int64_t nnz_ = 0;
    py::dtype dtype_;
    carr<int64_t> offsets_;

private:
    kpm_engine* h_ = nullptr;
    kpm_config cfg_{};
    py::object progress_ = py::none();

    py::array contiguous(py::object a) {
        return py::module_::import("numpy").attr("ascontiguousarray")(a, dtype_);
    }
    void set_shape(Csr const& c, py::object system_offsets) {
        rows_ = c.rows;
        dtype_ = c.dtype;
        nnz_ = c.indptr.size() > 0 ? c.indptr.data()[c.indptr.size() - 1] : 0;
        if (system_offsets.is_none()) {
            nsys_ = 1;
            offsets_ = carr<int64_t>(2);
            offsets_.mutable_data()[0] = 0;
            offsets_.mutable_data()[1] = rows_;
            has_offsets_ = false;
        } else {
            offsets_ = carr<int64_t>(system_offsets);
            nsys_ = static_cast<int32_t>(offsets_.size() - 1);
            has_offsets_ = true;
        }
    }
    int64_t const* offsets_ptr() const { return has_offsets_ ? offsets_.data() : nullptr; }
    bool has_offsets_ = false;
};

}  // namespace

PYBIND11_MODULE(_kpm_gb300, m) {
    m.doc() = "pybind11 binding of the GB300 KPM engine's C ABI (include/kpm_gb300.h)";
    py::class_<Engine>(m, "Engine")
        .def(py::init<py::object, py::dict, py::object>(), py::arg("hamiltonian"), py::arg("config") = py::dict(),
             py::arg("system_offsets") = py::none())
        .def_static(
            "from_engines",
            [](std::vector<Engine*> const& members, py::dict config) { return new Engine(members, config); },
            py::arg("engines"), py::arg("config") = py::dict(), py::return_value_policy::take_ownership)
        .def("close", &Engine::close)
        .def("set_hamiltonian", &Engine::set_hamiltonian, py::arg("hamiltonian"),
             py::arg("system_offsets") = py::none())
        .def("energy_bounds", &Engine::energy_bounds, py::arg("system") = 0)
        .def("scaling_factors", &Engine::scaling_factors, py::arg("system") = 0)
        .def("moments_diag", &Engine::moments_diag, py::arg("num_moments"), py::arg("starters"),
             py::arg("average") = false, py::arg("on_device_ptr") = py::none(), py::arg("num_vectors") = py::none())
        .def("calc_dos", &Engine::calc_dos, py::arg("energy"), py::arg("broadening"), py::arg("num_random"))
        .def("calc_ldos", &Engine::calc_ldos, py::arg("indices"), py::arg("energy"), py::arg("broadening"))
        .def("calc_ldos_batch", &Engine::calc_ldos_batch, py::arg("sites"), py::arg("energy"), py::arg("broadening"))
        .def("calc_greens", &Engine::calc_greens, py::arg("row"), py::arg("cols"), py::arg("energy"),
             py::arg("broadening"))
        .def("moments", &Engine::moments, py::arg("num_moments"), py::arg("alpha"), py::arg("beta") = py::none(),
             py::arg("op") = py::none())
        .def("calc_conductivity", &Engine::calc_conductivity, py::arg("left"), py::arg("right"),
             py::arg("chemical_potential"), py::arg("broadening"), py::arg("temperature"), py::arg("num_random"),
             py::arg("num_points"), py::arg("gemm_mode") = 0)
        .def("adjoint_diag", &Engine::adjoint_diag, py::arg("num_moments"), py::arg("starters"), py::arg("dl_dmu"),
             py::arg("checkpoint") = 0)
        .def("adjoint_conductivity", &Engine::adjoint_conductivity, py::arg("left"), py::arg("right"),
             py::arg("num_moments"), py::arg("starters"), py::arg("dl_dmu") = py::none())
        .def("set_progress_callback", &Engine::set_progress_callback, py::arg("callback"))
        .def("stats", &Engine::stats)
        .def("report", &Engine::report, py::arg("shortform") = false)
        .def("stream", &Engine::stream)
        .def_readonly("rows", &Engine::rows_)
        .def_readonly("num_systems", &Engine::nsys_)
        .def_readonly("system_offsets", &Engine::offsets_)
        .def_property_readonly("dtype", [](Engine const& e) { return e.dtype_; });

    m.def("round_num_moments", &round_num_moments, py::arg("n"));
    m.def(
        "damping_coefficients",
        [](std::string const& kernel, double param, int64_t num_moments) {
            auto out = carr<double>(static_cast<py::ssize_t>(num_moments));
            check(kpm_damping_coefficients(kernel_code(kernel), param, num_moments, out.mutable_data()));
            return out;
        },
        py::arg("kernel"), py::arg("param"), py::arg("num_moments"));
    m.def(
        "required_num_moments",
        [](std::string const& kernel, double param, double scaled_broadening) {
            return kpm_required_num_moments(kernel_code(kernel), param, scaled_broadening);
        },
        py::arg("kernel"), py::arg("param"), py::arg("scaled_broadening"));
}
