// epseon_cuda.hpp -- C++ host side of the `cuda` device: the same builder /
// task-handle object model as epseon_backend's gpu device, running on the
// libepseon_cuda C ABI (include/epscu.h).
//
// Reference classes mirrored (cpp/gpu/include/epseon/gpu/...):
//   PrecisionType / InvalidPrecisionTypeString   enums.hpp:19-42, enums.cpp:11-53
//   HardwareConfig                               task_configurator/hardware_config.hpp:12-76
//   MorsePotentialConfig / MorsePotentialGenerator / PotentialFileLoader
//                                                task_configurator/potential_source.hpp:13-234
//   VibwaAlgorithmConfig                         task_configurator/algorithm_config.hpp:76-199
//   TaskConfigurator<FP>                         task_configurator/task_configurator.hpp:16-133
//   TaskHandle<FP>                               task_handle.hpp:17-162
//   ComputeDeviceInterface                       device_interface.hpp:19-52
//   ComputeContext                               compute_context.cpp:41-117
//
// Units on this interface are the ones the reference's examples use: energies
// in cm^-1, distances in angstrom, masses in unified atomic mass units.  The C
// ABI underneath works in atomic units; the conversion constants are below.
#pragma once

#include <atomic>
#include <cstdint>
#include <memory>
#include <mutex>
#include <optional>
#include <stdexcept>
#include <stop_token>
#include <string>
#include <string_view>
#include <thread>
#include <vector>

#include "epscu.h"

namespace epseon::cuda::cpp {

// CODATA 2018
constexpr double kHartreeInvCm = 219474.6313632;
constexpr double kBohrAngstrom = 0.529177210903;
constexpr double kDaltonMe = 1822.888486209;

enum class PrecisionType { Float32, Float64, _Last };

class InvalidPrecisionTypeString : public std::exception {
    std::string message;

  public:
    explicit InvalidPrecisionTypeString(std::string_view sv);
    const char* what() const noexcept override { return message.c_str(); }
};

std::string toString(PrecisionType p);
PrecisionType toPrecisionType(std::string_view s);

template <typename FP>
PrecisionType getPrecisionType();

// ------------------------------------------------------------------ configs

struct HardwareConfig {
    uint32_t potential_buffer_size = 0;  // largest grid accepted (points)
    uint32_t group_size = 0;             // potentials per device batch (0: all)
    uint32_t allocation_block_size = 0;  // device arena block (bytes)
    bool operator==(const HardwareConfig&) const = default;
};

struct MorsePotentialConfig {
    double dissociation_energy = 0;        // cm^-1
    double equilibrium_bond_distance = 0;  // angstrom
    double well_width = 0;                 // 1/angstrom
    double min_r = 0, max_r = 0;           // angstrom
    uint32_t point_count = 0;
    bool operator==(const MorsePotentialConfig&) const = default;
};

struct LennardJonesPotentialConfig {
    double epsilon = 0;  // cm^-1 (well depth; shifted so the minimum is 0)
    double sigma = 0;    // angstrom
    double min_r = 0, max_r = 0;
    uint32_t point_count = 0;
    bool operator==(const LennardJonesPotentialConfig&) const = default;
};

// One tabulated curve on a uniform grid (values in cm^-1).
struct TabulatedPotential {
    std::vector<double> values;
    double min_r = 0, max_r = 0;
    std::optional<double> asymptote;  // default: the value at max_r
    bool operator==(const TabulatedPotential&) const = default;
};

// Everything the solver needs for one batch, in atomic units.
struct PotentialBatchData {
    std::vector<double> V;
    std::vector<int64_t> offsets;
    std::vector<int32_t> N;
    std::vector<double> r_min, r_max, asymptote;
};

class PotentialSource {
  public:
    virtual ~PotentialSource() = default;
    virtual bool equals(const PotentialSource& other) const = 0;
    virtual std::shared_ptr<PotentialSource> shared_clone() const = 0;
    virtual size_t size() const = 0;
    virtual uint32_t max_point_count() const = 0;
    // Tabulate potentials [first, first + count) (atomic units); ctx may be
    // used for device-side tabulation.
    virtual PotentialBatchData get_potential_data(epscu_ctx* ctx, size_t first, size_t count) const = 0;
};

class MorsePotentialGenerator : public PotentialSource {
  public:
    std::vector<MorsePotentialConfig> configurations;
    explicit MorsePotentialGenerator(std::vector<MorsePotentialConfig> c) : configurations(std::move(c)) {}
    bool equals(const PotentialSource& o) const override;
    std::shared_ptr<PotentialSource> shared_clone() const override {
        return std::make_shared<MorsePotentialGenerator>(*this);
    }
    size_t size() const override { return configurations.size(); }
    uint32_t max_point_count() const override;
    PotentialBatchData get_potential_data(epscu_ctx* ctx, size_t first, size_t count) const override;
};

class LennardJonesPotentialGenerator : public PotentialSource {
  public:
    std::vector<LennardJonesPotentialConfig> configurations;
    explicit LennardJonesPotentialGenerator(std::vector<LennardJonesPotentialConfig> c)
        : configurations(std::move(c)) {}
    bool equals(const PotentialSource& o) const override;
    std::shared_ptr<PotentialSource> shared_clone() const override {
        return std::make_shared<LennardJonesPotentialGenerator>(*this);
    }
    size_t size() const override { return configurations.size(); }
    uint32_t max_point_count() const override;
    PotentialBatchData get_potential_data(epscu_ctx* ctx, size_t first, size_t count) const override;
};

class TabulatedPotentialSource : public PotentialSource {
  public:
    std::vector<TabulatedPotential> curves;
    explicit TabulatedPotentialSource(std::vector<TabulatedPotential> c) : curves(std::move(c)) {}
    bool equals(const PotentialSource& o) const override;
    std::shared_ptr<PotentialSource> shared_clone() const override {
        return std::make_shared<TabulatedPotentialSource>(*this);
    }
    size_t size() const override { return curves.size(); }
    uint32_t max_point_count() const override;
    PotentialBatchData get_potential_data(epscu_ctx* ctx, size_t first, size_t count) const override;
};

// Reads two-column text files (r in angstrom, V in cm^-1; '#' comments).  A
// non-uniform grid is resampled onto the uniform grid with the same number of
// points by a natural cubic spline.  (The reference's PotentialFileLoader,
// potential_source.hpp:44-100, keeps file names and returns no data.)
class PotentialFileLoader : public PotentialSource {
  public:
    std::vector<std::string> file_names;
    explicit PotentialFileLoader(std::vector<std::string> f);
    bool equals(const PotentialSource& o) const override;
    std::shared_ptr<PotentialSource> shared_clone() const override {
        return std::make_shared<PotentialFileLoader>(*this);
    }
    size_t size() const override { return file_names.size(); }
    uint32_t max_point_count() const override;
    PotentialBatchData get_potential_data(epscu_ctx* ctx, size_t first, size_t count) const override;
    static TabulatedPotential load(const std::string& path);

  private:
    std::vector<TabulatedPotential> cache;
};

struct VibwaAlgorithmConfig {
    double mass_atom_0 = 0, mass_atom_1 = 0;  // Da
    double integration_step = 0;              // trial-energy spacing (cm^-1)
    double min_distance_to_asymptote = 0;     // cm^-1 below the asymptote
    uint32_t min_level = 0, max_level = 0;
    bool operator==(const VibwaAlgorithmConfig&) const = default;
    double reduced_mass_me() const { return mass_atom_0 * mass_atom_1 / (mass_atom_0 + mass_atom_1) * kDaltonMe; }
};

// ------------------------------------------------------------- configurator

template <typename FP>
class TaskConfigurator {
  public:
    std::shared_ptr<HardwareConfig> hardware_config;
    std::shared_ptr<PotentialSource> potential_source;
    std::shared_ptr<VibwaAlgorithmConfig> algorithm_config;
    bool want_wavefunctions = false;

    TaskConfigurator() = default;
    // deep copy (task_configurator.hpp:52-64)
    TaskConfigurator(const TaskConfigurator& o)
        : hardware_config(o.hardware_config ? std::make_shared<HardwareConfig>(*o.hardware_config) : nullptr),
          potential_source(o.potential_source ? o.potential_source->shared_clone() : nullptr),
          algorithm_config(o.algorithm_config ? std::make_shared<VibwaAlgorithmConfig>(*o.algorithm_config) : nullptr),
          want_wavefunctions(o.want_wavefunctions) {}

    TaskConfigurator& setHardwareConfig(const HardwareConfig& c) {
        hardware_config = std::make_shared<HardwareConfig>(c);
        return *this;
    }
    TaskConfigurator& setPotentialSource(const PotentialSource& s) {
        potential_source = s.shared_clone();
        return *this;
    }
    TaskConfigurator& setAlgorithmConfig(const VibwaAlgorithmConfig& c) {
        algorithm_config = std::make_shared<VibwaAlgorithmConfig>(c);
        return *this;
    }
    bool isConfigured() const { return hardware_config && potential_source && algorithm_config; }
};

// ----------------------------------------------------------------- results

struct TaskResults {
    std::vector<int32_t> n_total;                // bound levels below the cap, per potential
    std::vector<std::vector<double>> energies;   // cm^-1, levels min_level.. per potential
    std::vector<std::vector<int32_t>> nodes;
    std::vector<std::vector<int32_t>> status;
    std::vector<std::vector<double>> error_estimate;  // cm^-1
    std::vector<std::vector<double>> wavefunctions;   // [levels * N] per potential, angstrom^-1/2
    std::vector<int32_t> N;
    std::vector<double> r_min, r_max;             // angstrom
};

class ComputeDeviceInterface;

template <typename FP>
class TaskHandle : public std::enable_shared_from_this<TaskHandle<FP>> {
  public:
    TaskHandle(std::shared_ptr<ComputeDeviceInterface> dev, std::shared_ptr<TaskConfigurator<FP>> cfg)
        : device(std::move(dev)), config(std::move(cfg)) {}
    ~TaskHandle();

    void startWorker();
    bool isDone() const { return done.load(std::memory_order_acquire); }
    bool isStarted() const { return started.load(std::memory_order_acquire); }
    bool isRunning() const { return isStarted() && !isDone(); }
    bool cancel();
    void wait();
    std::string statusMessage() const;
    // results of a finished task; rethrows the worker's exception if it failed
    const TaskResults& results();

  private:
    static void run(std::stop_token st, TaskHandle* self);
    void execute(std::stop_token st);
    void setMessage(std::string m);

    std::shared_ptr<ComputeDeviceInterface> device;
    std::shared_ptr<TaskConfigurator<FP>> config;
    std::atomic<bool> done{false};
    std::atomic<bool> started{false};
    mutable std::mutex msg_mu;
    std::string message = "created";
    TaskResults res;
    std::exception_ptr error;
    // cancel() and the worker agree under run_mu: the context's flag is set
    // only while this task's solve runs (in_solve), and a request that came
    // after that solve had already finished is withdrawn by the worker
    std::mutex run_mu;
    bool in_solve = false;
    bool finished = false;
    std::jthread worker;
};

struct DeviceProperties {
    std::string api_version, driver_version, device_type, device_name;
    uint32_t vendor_id = 0x10DE, device_id = 0;
    std::vector<uint8_t> pipeline_cache_uuid;
    uint32_t max_compute_shared_memory_size = 0;
    uint32_t max_compute_work_group_count[3] = {0, 0, 0};
    uint32_t max_compute_work_group_invocations = 0;
    uint32_t max_compute_work_group_size = 0;
    int32_t ordinal = 0;
    int32_t sm_count = 0;
    int32_t compute_capability_major = 0, compute_capability_minor = 0;
};

struct MemoryHeap {
    uint64_t size = 0;
    std::vector<std::string> flags;
};
struct MemoryType {
    uint32_t heap_index = 0;
    std::vector<std::string> flags;
};
struct PhysicalDeviceInfo {
    DeviceProperties device_properties;
    std::vector<MemoryHeap> memory_heaps;
    std::vector<MemoryType> memory_types;
};

class ComputeDeviceInterface : public std::enable_shared_from_this<ComputeDeviceInterface> {
  public:
    explicit ComputeDeviceInterface(int32_t ordinal);
    ~ComputeDeviceInterface();
    template <typename FP>
    std::shared_ptr<TaskConfigurator<FP>> getTaskConfigurator() {
        return std::make_shared<TaskConfigurator<FP>>();
    }
    template <typename FP>
    std::shared_ptr<TaskHandle<FP>> submitTask(const std::shared_ptr<TaskConfigurator<FP>>& cfg) {
        if (!cfg || !cfg->isConfigured())
            throw std::runtime_error("TaskConfigurator wasn't fully configured before submitting for execution.");
        // the task owns a deep copy: later changes to the configurator do not leak in
        return std::make_shared<TaskHandle<FP>>(shared_from_this(), std::make_shared<TaskConfigurator<FP>>(*cfg));
    }
    epscu_ctx* context() const { return ctx; }
    int32_t ordinal() const { return ord; }
    // held by a task for the whole of each of its solves: tasks on one device
    // interface take the context in turn, so a task's cancel request reaches
    // the context only while that task's own solve holds it
    std::mutex& solveMutex() { return solve_mu; }

  private:
    int32_t ord;
    epscu_ctx* ctx = nullptr;
    std::mutex solve_mu;
};

class ComputeContext : public std::enable_shared_from_this<ComputeContext> {
  public:
    static std::shared_ptr<ComputeContext> create();
    std::string getApiVersion() const;
    std::vector<PhysicalDeviceInfo> getPhysicalDevicesInfo() const;
    // device_id: the PCI device ID reported in device_properties (as the
    // reference matches deviceID, compute_context.cpp:106-117); an ordinal is
    // accepted when no device has that ID.
    std::shared_ptr<ComputeDeviceInterface> getDeviceInterface(uint32_t device_id);
};

}  // namespace epseon::cuda::cpp
