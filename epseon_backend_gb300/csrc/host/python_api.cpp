// python_api.cpp -- the `_libepseon_cuda` Python module: the same classes,
// method names, argument names and error behaviour as the reference's
// `_libepseon_gpu` module (cpp/gpu/source/epseon/gpu/python/api.cpp:114-494,
// python/epseon_backend/device/gpu/_libepseon_gpu.pyi:81-180), on the CUDA
// solver.  Additions (absent from the reference): LennardJonesPotentialConfig,
// set_lj_potential, set_tabulated_potential, set_potential_files,
// set_wavefunction_output, TaskHandle.cancel/is_running/get_results.
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <optional>
#include <variant>

#include "epseon_cuda.hpp"

namespace py = pybind11;
using namespace epseon::cuda;

namespace {

template <typename FP>
class PyTaskHandle {
  public:
    std::shared_ptr<cpp::TaskHandle<FP>> h;
    explicit PyTaskHandle(std::shared_ptr<cpp::TaskHandle<FP>> h_) : h(std::move(h_)) {
        if (!h->isRunning()) h->startWorker();
    }
    std::string get_status_message() { return h->statusMessage(); }
    bool is_done() { return h->isDone(); }
    bool is_running() { return h->isRunning(); }
    bool cancel() { return h->cancel(); }
    void wait() {
        py::gil_scoped_release nogil;
        h->wait();
    }
    py::dict get_results() {
        const cpp::TaskResults* r;
        {
            py::gil_scoped_release nogil;
            r = &h->results();
        }
        py::dict d;
        py::list energies, nodes, status, err, psi, grids;
        for (size_t i = 0; i < r->energies.size(); ++i) {
            energies.append(py::array_t<double>(r->energies[i].size(), r->energies[i].data()));
            nodes.append(py::array_t<int32_t>(r->nodes[i].size(), r->nodes[i].data()));
            status.append(py::array_t<int32_t>(r->status[i].size(), r->status[i].data()));
            err.append(py::array_t<double>(r->error_estimate[i].size(), r->error_estimate[i].data()));
            if (!r->wavefunctions[i].empty()) {
                const py::ssize_t rows = (py::ssize_t)r->energies[i].size(), cols = r->N[i];
                py::array_t<double> a({rows, cols});
                std::memcpy(a.mutable_data(), r->wavefunctions[i].data(), sizeof(double) * rows * cols);
                psi.append(a);
            } else {
                psi.append(py::none());
            }
            py::array_t<double> g(r->N[i]);
            auto* gp = g.mutable_data();
            const double hh = (r->r_max[i] - r->r_min[i]) / (double)(r->N[i] - 1);
            for (int32_t j = 0; j < r->N[i]; ++j) gp[j] = r->r_min[i] + hh * j;
            grids.append(g);
        }
        d["energies"] = energies;
        d["nodes"] = nodes;
        d["status"] = status;
        d["error_estimate"] = err;
        d["wavefunctions"] = psi;
        d["r"] = grids;
        d["n_total"] = py::array_t<int32_t>(r->n_total.size(), r->n_total.data());
        d["units"] = py::dict(py::arg("energy") = "cm^-1", py::arg("r") = "angstrom",
                              py::arg("psi") = "angstrom^-1/2");
        return d;
    }
};

using PyTaskHandleVariant = std::variant<PyTaskHandle<float>, PyTaskHandle<double>>;

template <typename FP>
class PyTaskConfigurator {
  public:
    std::shared_ptr<cpp::TaskConfigurator<FP>> c;
    explicit PyTaskConfigurator(std::shared_ptr<cpp::TaskConfigurator<FP>> c_) : c(std::move(c_)) {}

    PyTaskConfigurator& set_hardware_config(uint32_t potential_buffer_size, uint32_t group_size,
                                            uint32_t allocation_block_size) {
        c->setHardwareConfig({potential_buffer_size, group_size, allocation_block_size});
        return *this;
    }
    // api.hpp:169-218; equal point counts are required as in the reference
    // (the reference's duplicate-entry bug, api.hpp:175-202, is not copied)
    PyTaskConfigurator& set_morse_potential(const std::vector<cpp::MorsePotentialConfig>& configs) {
        std::optional<uint32_t> pc;
        for (const auto& e : configs) {
            if (pc && *pc != e.point_count)
                throw std::runtime_error("All Morse potentials must have same point count, but previous ones had " +
                                         std::to_string(*pc) + " and current one has " +
                                         std::to_string(e.point_count) + ".");
            pc = e.point_count;
        }
        c->setPotentialSource(cpp::MorsePotentialGenerator(configs));
        return *this;
    }
    PyTaskConfigurator& set_lj_potential(const std::vector<cpp::LennardJonesPotentialConfig>& configs) {
        c->setPotentialSource(cpp::LennardJonesPotentialGenerator(configs));
        return *this;
    }
    PyTaskConfigurator& set_tabulated_potential(const std::vector<py::array_t<double, py::array::c_style |
                                                                                  py::array::forcecast>>& values,
                                                double min_r, double max_r, std::optional<double> asymptote) {
        std::vector<cpp::TabulatedPotential> curves;
        for (const auto& a : values) {
            cpp::TabulatedPotential t;
            t.values.assign(a.data(), a.data() + a.size());
            t.min_r = min_r;
            t.max_r = max_r;
            t.asymptote = asymptote;
            curves.push_back(std::move(t));
        }
        c->setPotentialSource(cpp::TabulatedPotentialSource(std::move(curves)));
        return *this;
    }
    PyTaskConfigurator& set_potential_files(const std::vector<std::string>& files) {
        c->setPotentialSource(cpp::PotentialFileLoader(files));
        return *this;
    }
    PyTaskConfigurator& set_vibwa_algorithm(double mass_atom_0, double mass_atom_1, double integration_step,
                                            double min_distance_to_asymptote, uint32_t min_level,
                                            uint32_t max_level) {
        c->setAlgorithmConfig(
            {mass_atom_0, mass_atom_1, integration_step, min_distance_to_asymptote, min_level, max_level});
        return *this;
    }
    PyTaskConfigurator& set_wavefunction_output(bool enabled) {
        c->want_wavefunctions = enabled;
        return *this;
    }
    bool is_configured() const { return c->isConfigured(); }
};

using PyConfiguratorVariant = std::variant<PyTaskConfigurator<float>, PyTaskConfigurator<double>>;

class PyComputeDeviceInterface {
  public:
    std::shared_ptr<cpp::ComputeDeviceInterface> d;
    explicit PyComputeDeviceInterface(std::shared_ptr<cpp::ComputeDeviceInterface> d_) : d(std::move(d_)) {}
    PyConfiguratorVariant get_task_configurator(const std::string& precision) {
        cpp::PrecisionType p;
        try {
            p = cpp::toPrecisionType(precision);
        } catch (const cpp::InvalidPrecisionTypeString& e) {
            throw py::value_error(e.what());
        }
        if (p == cpp::PrecisionType::Float32) return PyTaskConfigurator<float>(d->getTaskConfigurator<float>());
        return PyTaskConfigurator<double>(d->getTaskConfigurator<double>());
    }
    template <typename FP>
    PyTaskHandleVariant submit_task(const PyTaskConfigurator<FP>& cfg) {
        if (!cfg.is_configured())
            throw std::runtime_error("TaskConfigurator submitted for execution before fully configured.");
        return PyTaskHandle<FP>(d->submitTask<FP>(cfg.c));
    }
};

class PyComputeContext {
  public:
    std::shared_ptr<cpp::ComputeContext> ctx;
    static PyComputeContext create() { return PyComputeContext{cpp::ComputeContext::create()}; }
    std::string get_vulkan_version() { return ctx->getApiVersion(); }
    std::vector<cpp::PhysicalDeviceInfo> get_physical_device_info() { return ctx->getPhysicalDevicesInfo(); }
    PyComputeDeviceInterface get_device_interface(uint32_t device_id) {
        return PyComputeDeviceInterface{ctx->getDeviceInterface(device_id)};
    }
};

struct SparseProperties {};

template <typename FP, typename C>
void bind_configurator(py::module_& m, const char* name) {
    using T = PyTaskConfigurator<FP>;
    py::class_<T>(m, name)
        .def("set_hardware_config", &T::set_hardware_config, py::arg("potential_buffer_size"),
             py::arg("group_size"), py::arg("allocation_block_size"),
             "Set hardware configuration for a GPU compute task.", py::return_value_policy::reference)
        .def("set_morse_potential", &T::set_morse_potential, py::arg("configurations"),
             "Set potential data source configuration for GPU compute task.", py::return_value_policy::reference)
        .def("set_lj_potential", &T::set_lj_potential, py::arg("configurations"),
             "Use shifted Lennard-Jones 12-6 potentials (minimum 0, asymptote epsilon).",
             py::return_value_policy::reference)
        .def("set_tabulated_potential", &T::set_tabulated_potential, py::arg("values"), py::arg("min_r"),
             py::arg("max_r"), py::arg("asymptote") = py::none(),
             "Use tabulated curves (cm^-1) on the uniform grid [min_r, max_r] (angstrom).",
             py::return_value_policy::reference)
        .def("set_potential_files", &T::set_potential_files, py::arg("file_names"),
             "Load two-column (r [angstrom], V [cm^-1]) potential files.", py::return_value_policy::reference)
        .def("set_vibwa_algorithm", &T::set_vibwa_algorithm, py::arg("mass_atom_0"), py::arg("mass_atom_1"),
             py::arg("integration_step"), py::arg("min_distance_to_asymptote"), py::arg("min_level"),
             py::arg("max_level"), "Set algorithm configuration for a GPU compute task.",
             py::return_value_policy::reference)
        .def("set_wavefunction_output", &T::set_wavefunction_output, py::arg("enabled"),
             "Also return the normalised wavefunctions of every level.", py::return_value_policy::reference)
        .def("is_configured", &T::is_configured,
             "Check if this instance is fully configured, i.e. it has been assigned a valid hardware "
             "configuration, potential source and algorithm config.")
        .doc() = "Builder for configuring GPU compute task.";
}

template <typename FP>
void bind_handle(py::module_& m, const char* name) {
    using T = PyTaskHandle<FP>;
    py::class_<T>(m, name)
        .def("get_status_message", &T::get_status_message, "Get status message explaining current execution stage.")
        .def("is_done", &T::is_done, "Check if task already finished execution.")
        .def("is_running", &T::is_running, "Check if task is still running.")
        .def("cancel", &T::cancel, "Request cooperative cancellation of the task.")
        .def("wait", &T::wait, "Block and wait for task to finish.")
        .def("get_results", &T::get_results,
             "Levels of every potential: energies (cm^-1), nodes, status bits, error estimates, "
             "wavefunctions (when enabled) and the radial grids.")
        .doc() = "Handle object for referencing GPU compute task.";
}

}  // namespace

PYBIND11_MODULE(_libepseon_cuda, m) {
    m.doc() = "Sub package for interacting with the CUDA (GB300) compute device.";

    py::class_<SparseProperties>(m, "PhysicalDeviceSparseProperties").doc() = "Sparse resource properties (none on CUDA).";

    py::class_<cpp::DeviceProperties>(m, "PhysicalDeviceProperties")
        .def_readonly("api_version", &cpp::DeviceProperties::api_version)
        .def_readonly("driver_version", &cpp::DeviceProperties::driver_version)
        .def_readonly("vendor_id", &cpp::DeviceProperties::vendor_id)
        .def_readonly("device_id", &cpp::DeviceProperties::device_id)
        .def_readonly("device_type", &cpp::DeviceProperties::device_type)
        .def_readonly("device_name", &cpp::DeviceProperties::device_name)
        .def_property_readonly("pipeline_cache_uuid",
                               [](const cpp::DeviceProperties& p) {
                                   return std::vector<int>(p.pipeline_cache_uuid.begin(), p.pipeline_cache_uuid.end());
                               })
        .def_property_readonly("limits", [](const cpp::DeviceProperties& p) { return p; })
        .def_property_readonly("sparse_properties", [](const cpp::DeviceProperties&) { return SparseProperties{}; })
        .def_readonly("ordinal", &cpp::DeviceProperties::ordinal)
        .def_readonly("sm_count", &cpp::DeviceProperties::sm_count)
        .def_property_readonly("max_compute_shared_memory_size",
                               [](const cpp::DeviceProperties& p) { return p.max_compute_shared_memory_size; })
        .def_property_readonly("max_compute_work_group_count",
                               [](const cpp::DeviceProperties& p) {
                                   return py::make_tuple(p.max_compute_work_group_count[0],
                                                         p.max_compute_work_group_count[1],
                                                         p.max_compute_work_group_count[2]);
                               })
        .def_property_readonly("max_compute_work_group_invocations",
                               [](const cpp::DeviceProperties& p) { return p.max_compute_work_group_invocations; })
        .def_property_readonly("max_compute_work_group_size",
                               [](const cpp::DeviceProperties& p) { return p.max_compute_work_group_size; })
        .doc() = "Properties of a CUDA device (limits are exposed on the same object).";

    py::class_<cpp::MemoryHeap>(m, "MemoryHeap")
        .def_readonly("size", &cpp::MemoryHeap::size)
        .def_readonly("flags", &cpp::MemoryHeap::flags);
    py::class_<cpp::MemoryType>(m, "MemoryType")
        .def_readonly("heap_index", &cpp::MemoryType::heap_index)
        .def_readonly("flags", &cpp::MemoryType::flags);
    py::class_<cpp::PhysicalDeviceInfo>(m, "PhysicalDeviceInfo")
        .def_readonly("device_properties", &cpp::PhysicalDeviceInfo::device_properties)
        .def_property_readonly("memory_properties", [](const cpp::PhysicalDeviceInfo& d) { return d; })
        .def_readonly("memory_heaps", &cpp::PhysicalDeviceInfo::memory_heaps)
        .def_readonly("memory_types", &cpp::PhysicalDeviceInfo::memory_types)
        .doc() = "Container for CUDA device info.";

    bind_handle<float>(m, "TaskHandleFloat32");
    bind_handle<double>(m, "TaskHandleFloat64");

    py::class_<cpp::MorsePotentialConfig>(m, "MorsePotentialConfig")
        .def(py::init([](double De, double re, double a, double r0, double r1, uint32_t n) {
                 return cpp::MorsePotentialConfig{De, re, a, r0, r1, n};
             }),
             py::arg("dissociation_energy"), py::arg("equilibrium_bond_distance"), py::arg("well_width"),
             py::arg("min_r"), py::arg("max_r"), py::arg("point_count"),
             "Create instance of MorsePotentialConfig class.")
        .def_readonly("dissociation_energy", &cpp::MorsePotentialConfig::dissociation_energy)
        .def_readonly("equilibrium_bond_distance", &cpp::MorsePotentialConfig::equilibrium_bond_distance)
        .def_readonly("well_width", &cpp::MorsePotentialConfig::well_width)
        .def_readonly("min_r", &cpp::MorsePotentialConfig::min_r)
        .def_readonly("max_r", &cpp::MorsePotentialConfig::max_r)
        .def_readonly("point_count", &cpp::MorsePotentialConfig::point_count)
        .doc() = "Configuration of single Morse potential curve.";

    py::class_<cpp::LennardJonesPotentialConfig>(m, "LennardJonesPotentialConfig")
        .def(py::init([](double eps, double sigma, double r0, double r1, uint32_t n) {
                 return cpp::LennardJonesPotentialConfig{eps, sigma, r0, r1, n};
             }),
             py::arg("epsilon"), py::arg("sigma"), py::arg("min_r"), py::arg("max_r"), py::arg("point_count"))
        .doc() = "Configuration of a shifted Lennard-Jones 12-6 curve.";

    bind_configurator<float, void>(m, "TaskConfiguratorFloat32");
    bind_configurator<double, void>(m, "TaskConfiguratorFloat64");

    py::class_<PyComputeDeviceInterface>(m, "ComputeDeviceInterface")
        .def("get_task_configurator", &PyComputeDeviceInterface::get_task_configurator,
             "Get builder instance for configuring GPU compute task.")
        .def("submit_task", &PyComputeDeviceInterface::submit_task<float>,
             "Submit task for execution. Will raise RuntimeError upon receiving not fully configured "
             "TaskConfigurator.")
        .def("submit_task", &PyComputeDeviceInterface::submit_task<double>,
             "Submit task for execution. Will raise RuntimeError upon receiving not fully configured "
             "TaskConfigurator.")
        .doc() = "Interface to particular CUDA device.";

    py::class_<PyComputeContext>(m, "EpseonComputeContext")
        .def_static("create", &PyComputeContext::create, "Create instance of EpseonComputeContext object.")
        .def("get_vulkan_version", &PyComputeContext::get_vulkan_version,
             "CUDA driver and runtime versions as 'driver_major.driver_minor.runtime_major.runtime_minor' (the "
             "name is kept for drop-in compatibility).")
        .def("get_physical_device_info", &PyComputeContext::get_physical_device_info,
             "Get information about available CUDA devices.")
        .def("get_device_interface", &PyComputeContext::get_device_interface,
             "Get interface for running algorithms on a CUDA device.")
        .doc() = "CUDA compute context handle.";
}
