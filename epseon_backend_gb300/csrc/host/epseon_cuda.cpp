// epseon_cuda.cpp -- implementation of the C++ host side of the `cuda` device.
#include "epseon_cuda.hpp"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>

namespace epseon::cuda::cpp {

namespace {

std::string abi_error(const char* what, epscu_status st) {
    return std::string(what) + " failed (" + std::to_string(st) + "): " + epscu_last_error();
}

void check(const char* what, epscu_status st) {
    if (st != EPSCU_OK) throw std::runtime_error(abi_error(what, st));
}

double to_hartree(double cm) { return cm / kHartreeInvCm; }
double to_bohr(double ang) { return ang / kBohrAngstrom; }

// natural cubic spline through (x_k, y_k) evaluated at xs (x strictly increasing)
std::vector<double> spline_resample(const std::vector<double>& x, const std::vector<double>& y,
                                    const std::vector<double>& xs) {
    const size_t n = x.size();
    std::vector<double> M(n, 0.0);
    if (n >= 3) {
        std::vector<double> c(n, 0.0), d(n, 0.0);
        for (size_t i = 1; i + 1 < n; ++i) {
            const double h0 = x[i] - x[i - 1], h1 = x[i + 1] - x[i];
            const double a = h0, b = 2.0 * (h0 + h1), cc = h1;
            const double r = 6.0 * ((y[i + 1] - y[i]) / h1 - (y[i] - y[i - 1]) / h0);
            const double den = b - a * c[i - 1];
            c[i] = cc / den;
            d[i] = (r - a * d[i - 1]) / den;
        }
        for (size_t i = n - 2; i >= 1; --i) {
            M[i] = d[i] - c[i] * M[i + 1];
            if (i == 1) break;
        }
    }
    std::vector<double> out(xs.size());
    size_t k = 0;
    for (size_t j = 0; j < xs.size(); ++j) {
        const double t = xs[j];
        while (k + 2 < n && x[k + 1] < t) ++k;
        const double h = x[k + 1] - x[k];
        const double A = (x[k + 1] - t) / h, B = (t - x[k]) / h;
        out[j] = A * y[k] + B * y[k + 1] + ((A * A * A - A) * M[k] + (B * B * B - B) * M[k + 1]) * h * h / 6.0;
    }
    return out;
}

}  // namespace

InvalidPrecisionTypeString::InvalidPrecisionTypeString(std::string_view sv)
    : message("Invalid PrecisionType literal in string: \"" + std::string(sv) + "\"") {}

std::string toString(PrecisionType p) {
    switch (p) {
        case PrecisionType::Float32:
            return "Float32";
        case PrecisionType::Float64:
            return "Float64";
        default:
            throw std::runtime_error("Unreachable");
    }
}

PrecisionType toPrecisionType(std::string_view s) {
    std::string low(s);
    std::transform(low.begin(), low.end(), low.begin(), [](unsigned char c) { return (char)std::tolower(c); });
    if (low == "float32") return PrecisionType::Float32;
    if (low == "float64") return PrecisionType::Float64;
    throw InvalidPrecisionTypeString(low);
}

template <>
PrecisionType getPrecisionType<float>() {
    return PrecisionType::Float32;
}
template <>
PrecisionType getPrecisionType<double>() {
    return PrecisionType::Float64;
}

// ------------------------------------------------------------ potential sources

bool MorsePotentialGenerator::equals(const PotentialSource& o) const {
    auto* x = dynamic_cast<const MorsePotentialGenerator*>(&o);
    return x && x->configurations == configurations;
}

uint32_t MorsePotentialGenerator::max_point_count() const {
    uint32_t m = 0;
    for (auto& c : configurations) m = std::max(m, c.point_count);
    return m;
}

static PotentialBatchData tabulate_on_device(epscu_ctx* ctx, const std::vector<int32_t>& kind,
                                             const std::vector<double>& params, const std::vector<int32_t>& N,
                                             const std::vector<double>& r0, const std::vector<double>& r1,
                                             const std::vector<double>& asym) {
    PotentialBatchData d;
    const size_t n = kind.size();
    d.N = N;
    d.r_min = r0;
    d.r_max = r1;
    d.asymptote = asym;
    d.offsets.resize(n);
    int64_t total = 0;
    for (size_t i = 0; i < n; ++i) {
        d.offsets[i] = total;
        total += N[i];
    }
    d.V.assign((size_t)total, 0.0);
    epscu_opts o{};
    check("epscu_tabulate", epscu_tabulate(ctx, (int32_t)n, kind.data(), params.data(), d.offsets.data(), N.data(),
                                           r0.data(), r1.data(), 1024, d.V.data(), &o));
    return d;
}

PotentialBatchData MorsePotentialGenerator::get_potential_data(epscu_ctx* ctx, size_t first, size_t count) const {
    std::vector<int32_t> kind, N;
    std::vector<double> params, r0, r1, asym;
    for (size_t i = first; i < first + count; ++i) {
        const auto& c = configurations[i];
        kind.push_back(EPSCU_KIND_MORSE);
        double p[12] = {to_hartree(c.dissociation_energy), c.well_width * kBohrAngstrom,
                        to_bohr(c.equilibrium_bond_distance)};
        params.insert(params.end(), p, p + 12);
        N.push_back((int32_t)c.point_count);
        r0.push_back(to_bohr(c.min_r));
        r1.push_back(to_bohr(c.max_r));
        asym.push_back(to_hartree(c.dissociation_energy));
    }
    return tabulate_on_device(ctx, kind, params, N, r0, r1, asym);
}

bool LennardJonesPotentialGenerator::equals(const PotentialSource& o) const {
    auto* x = dynamic_cast<const LennardJonesPotentialGenerator*>(&o);
    return x && x->configurations == configurations;
}

uint32_t LennardJonesPotentialGenerator::max_point_count() const {
    uint32_t m = 0;
    for (auto& c : configurations) m = std::max(m, c.point_count);
    return m;
}

PotentialBatchData LennardJonesPotentialGenerator::get_potential_data(epscu_ctx* ctx, size_t first,
                                                                      size_t count) const {
    std::vector<int32_t> kind, N;
    std::vector<double> params, r0, r1, asym;
    for (size_t i = first; i < first + count; ++i) {
        const auto& c = configurations[i];
        kind.push_back(EPSCU_KIND_LJ);
        double p[12] = {to_hartree(c.epsilon), to_bohr(c.sigma)};
        params.insert(params.end(), p, p + 12);
        N.push_back((int32_t)c.point_count);
        r0.push_back(to_bohr(c.min_r));
        r1.push_back(to_bohr(c.max_r));
        asym.push_back(to_hartree(c.epsilon));
    }
    return tabulate_on_device(ctx, kind, params, N, r0, r1, asym);
}

bool TabulatedPotentialSource::equals(const PotentialSource& o) const {
    auto* x = dynamic_cast<const TabulatedPotentialSource*>(&o);
    return x && x->curves == curves;
}

uint32_t TabulatedPotentialSource::max_point_count() const {
    size_t m = 0;
    for (auto& c : curves) m = std::max(m, c.values.size());
    return (uint32_t)m;
}

static PotentialBatchData from_curves(const std::vector<TabulatedPotential>& curves, size_t first, size_t count) {
    PotentialBatchData d;
    int64_t total = 0;
    for (size_t i = first; i < first + count; ++i) {
        const auto& c = curves[i];
        d.offsets.push_back(total);
        d.N.push_back((int32_t)c.values.size());
        d.r_min.push_back(to_bohr(c.min_r));
        d.r_max.push_back(to_bohr(c.max_r));
        const double asym = c.asymptote ? *c.asymptote : (c.values.empty() ? 0.0 : c.values.back());
        d.asymptote.push_back(to_hartree(asym));
        for (double v : c.values) d.V.push_back(to_hartree(v));
        total += (int64_t)c.values.size();
    }
    return d;
}

PotentialBatchData TabulatedPotentialSource::get_potential_data(epscu_ctx*, size_t first, size_t count) const {
    return from_curves(curves, first, count);
}

PotentialFileLoader::PotentialFileLoader(std::vector<std::string> f) : file_names(std::move(f)) {
    for (auto& name : file_names) cache.push_back(load(name));
}

bool PotentialFileLoader::equals(const PotentialSource& o) const {
    auto* x = dynamic_cast<const PotentialFileLoader*>(&o);
    return x && x->file_names == file_names;
}

uint32_t PotentialFileLoader::max_point_count() const {
    size_t m = 0;
    for (auto& c : cache) m = std::max(m, c.values.size());
    return (uint32_t)m;
}

TabulatedPotential PotentialFileLoader::load(const std::string& path) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error("cannot open potential file: " + path);
    std::vector<double> r, v;
    std::string line;
    size_t lineno = 0;
    while (std::getline(in, line)) {
        ++lineno;
        const auto hash = line.find('#');
        if (hash != std::string::npos) line.resize(hash);
        for (char& ch : line)
            if (ch == ',' || ch == ';' || ch == '\t') ch = ' ';
        std::istringstream ss(line);
        double a, b;
        if (!(ss >> a)) continue;  // blank line
        if (!(ss >> b)) throw std::runtime_error(path + ":" + std::to_string(lineno) + ": expected two columns");
        r.push_back(a);
        v.push_back(b);
    }
    if (r.size() < 5) throw std::runtime_error(path + ": fewer than 5 points");
    for (size_t i = 1; i < r.size(); ++i)
        if (!(r[i] > r[i - 1])) throw std::runtime_error(path + ": r must be strictly increasing");
    TabulatedPotential t;
    t.min_r = r.front();
    t.max_r = r.back();
    const size_t n = r.size();
    const double h = (t.max_r - t.min_r) / (double)(n - 1);
    bool uniform = true;
    for (size_t i = 0; i < n && uniform; ++i)
        if (std::fabs(r[i] - (t.min_r + h * (double)i)) > 1e-9 * std::max(1.0, std::fabs(t.max_r))) uniform = false;
    if (uniform) {
        t.values = v;
    } else {
        std::vector<double> xs(n);
        for (size_t i = 0; i < n; ++i) xs[i] = t.min_r + h * (double)i;
        xs.back() = t.max_r;
        t.values = spline_resample(r, v, xs);
    }
    return t;
}

PotentialBatchData PotentialFileLoader::get_potential_data(epscu_ctx*, size_t first, size_t count) const {
    return from_curves(cache, first, count);
}

// ------------------------------------------------------------------ devices

ComputeDeviceInterface::ComputeDeviceInterface(int32_t ordinal) : ord(ordinal) {
    check("epscu_create", epscu_create(ordinal, &ctx));
}

ComputeDeviceInterface::~ComputeDeviceInterface() {
    if (ctx) epscu_destroy(ctx);
}

std::shared_ptr<ComputeContext> ComputeContext::create() {
    int32_t n = 0;
    const epscu_status st = epscu_device_count(&n);
    if (st != EPSCU_OK || n < 1) throw std::runtime_error("Failed to create EpseonComputeContext: no CUDA device");
    return std::make_shared<ComputeContext>();
}

std::string ComputeContext::getApiVersion() const {
    epscu_device_info info{};
    check("epscu_get_device_info", epscu_get_device_info(0, &info));
    const int dv = info.driver_version, rv = info.runtime_version;
    return std::to_string(dv / 1000) + "." + std::to_string((dv % 1000) / 10) + "." + std::to_string(rv / 1000) +
           "." + std::to_string((rv % 1000) / 10);
}

std::vector<PhysicalDeviceInfo> ComputeContext::getPhysicalDevicesInfo() const {
    int32_t n = 0;
    check("epscu_device_count", epscu_device_count(&n));
    std::vector<PhysicalDeviceInfo> out;
    for (int32_t i = 0; i < n; ++i) {
        epscu_device_info info{};
        check("epscu_get_device_info", epscu_get_device_info(i, &info));
        PhysicalDeviceInfo d;
        auto& p = d.device_properties;
        p.api_version = std::to_string(info.runtime_version / 1000) + "." +
                        std::to_string((info.runtime_version % 1000) / 10) + ".0";
        p.driver_version = std::to_string(info.driver_version / 1000) + "." +
                           std::to_string((info.driver_version % 1000) / 10) + ".0";
        p.vendor_id = 0x10DE;
        p.device_id = (uint32_t)info.pci_device_id;
        p.device_type = "DISCRETE_GPU";
        p.device_name = info.name;
        p.pipeline_cache_uuid.assign(info.uuid, info.uuid + 16);
        p.max_compute_shared_memory_size = (uint32_t)info.shared_mem_per_block_optin;
        for (int k = 0; k < 3; ++k) p.max_compute_work_group_count[k] = (uint32_t)info.max_grid_dim[k];
        p.max_compute_work_group_invocations = (uint32_t)info.max_threads_per_block;
        p.max_compute_work_group_size = (uint32_t)info.max_block_dim[0];
        p.ordinal = i;
        p.sm_count = info.sm_count;
        p.compute_capability_major = info.cc_major;
        p.compute_capability_minor = info.cc_minor;
        d.memory_heaps.push_back({(uint64_t)info.total_global_mem, {"DEVICE_LOCAL"}});
        d.memory_types.push_back({0, {"DEVICE_LOCAL"}});
        out.push_back(std::move(d));
    }
    return out;
}

std::shared_ptr<ComputeDeviceInterface> ComputeContext::getDeviceInterface(uint32_t device_id) {
    const auto devs = getPhysicalDevicesInfo();
    for (const auto& d : devs)
        if (d.device_properties.device_id == device_id)
            return std::make_shared<ComputeDeviceInterface>(d.device_properties.ordinal);
    if (device_id < devs.size()) return std::make_shared<ComputeDeviceInterface>((int32_t)device_id);
    throw std::runtime_error("Device not available.");
}

// -------------------------------------------------------------------- tasks

template <typename FP>
TaskHandle<FP>::~TaskHandle() {
    if (worker.joinable()) {
        cancel();
        worker.join();
    }
}

template <typename FP>
void TaskHandle<FP>::setMessage(std::string m) {
    std::lock_guard<std::mutex> g(msg_mu);
    message = std::move(m);
}

template <typename FP>
std::string TaskHandle<FP>::statusMessage() const {
    std::lock_guard<std::mutex> g(msg_mu);
    return message;
}

template <typename FP>
void TaskHandle<FP>::startWorker() {
    if (isRunning()) throw std::runtime_error("One worker is already running, can't start another one.");
    done.store(false, std::memory_order_release);
    started.store(true, std::memory_order_release);
    setMessage("queued");
    worker = std::jthread(run, this);
}

template <typename FP>
void TaskHandle<FP>::run(std::stop_token st, TaskHandle* self) {
    try {
        self->execute(st);
    } catch (...) {
        self->error = std::current_exception();
        try {
            std::rethrow_exception(self->error);
        } catch (const std::exception& e) {
            self->setMessage(std::string("failed: ") + e.what());
        } catch (...) {
            self->setMessage("failed");
        }
    }
    {
        std::lock_guard<std::mutex> g(self->run_mu);
        self->finished = true;
    }
    self->done.store(true, std::memory_order_release);
}

template <typename FP>
bool TaskHandle<FP>::cancel() {
    if (!isStarted()) return false;
    std::lock_guard<std::mutex> g(run_mu);
    if (finished) return false;
    const bool r = worker.request_stop();
    // the device solve in flight polls the context's flag; between solves the
    // worker sees the stop request before it starts the next one
    if (in_solve && device && device->context()) epscu_cancel(device->context());
    return r;
}

template <typename FP>
void TaskHandle<FP>::wait() {
    if (worker.joinable()) worker.join();
}

template <typename FP>
const TaskResults& TaskHandle<FP>::results() {
    wait();
    if (error) std::rethrow_exception(error);
    return res;
}

template <typename FP>
void TaskHandle<FP>::execute(std::stop_token st) {
    const auto& cfg = *config;
    const auto& hw = *cfg.hardware_config;
    const auto& alg = *cfg.algorithm_config;
    const auto& src = *cfg.potential_source;
    epscu_ctx* ctx = device->context();
    if (hw.potential_buffer_size && src.max_point_count() > hw.potential_buffer_size)
        throw std::runtime_error("point_count " + std::to_string(src.max_point_count()) +
                                 " exceeds potential_buffer_size " + std::to_string(hw.potential_buffer_size));
    if (!(alg.mass_atom_0 > 0) || !(alg.mass_atom_1 > 0)) throw std::runtime_error("atom masses must be positive");
    if (alg.max_level < alg.min_level) throw std::runtime_error("max_level < min_level");
    if (hw.allocation_block_size) epscu_set_arena_block(ctx, hw.allocation_block_size);
    const double mu = alg.reduced_mass_me();
    const int method = getPrecisionType<FP>() == PrecisionType::Float32 ? EPSCU_METHOD_FAST_FP32C
                                                                       : EPSCU_METHOD_PLAIN_FP64;
    const size_t total = src.size();
    const size_t group = hw.group_size ? hw.group_size : total;
    const int32_t cap = (int32_t)(alg.max_level - alg.min_level + 1);
    const double dist = to_hartree(alg.min_distance_to_asymptote);
    // the widest energy window of a group's potentials (cap - min V)
    auto span_of = [&](const PotentialBatchData& d) {
        double span = 0.0;
        for (size_t i = 0; i < d.N.size(); ++i) {
            const int64_t o = d.offsets[i];
            double vmin = d.V[o];
            for (int32_t j = 0; j < d.N[i]; ++j) vmin = std::min(vmin, d.V[o + j]);
            span = std::max(span, d.asymptote[i] - dist - vmin);
        }
        return span;
    };
    // The trial grid is the task's, not the group's: n_trial follows the
    // widest window of the whole task, so splitting a task into groups
    // (HardwareConfig::group_size) changes no result.  With several groups
    // the potentials are tabulated once more for this.
    double task_span = -1.0;
    if (group < total) {
        task_span = 0.0;
        for (size_t first = 0; first < total && !st.stop_requested(); first += group)
            task_span = std::max(task_span, span_of(src.get_potential_data(ctx, first, std::min(group, total - first))));
    }
    res = TaskResults{};
    for (size_t first = 0; first < total; first += group) {
        if (st.stop_requested()) {
            setMessage("cancelled");
            return;
        }
        const size_t count = std::min(group, total - first);
        setMessage("tabulating potentials " + std::to_string(first) + ".." + std::to_string(first + count));
        PotentialBatchData d = src.get_potential_data(ctx, first, count);
        const int n = (int)count;
        std::vector<double> mus(n, mu), cap_e(n);
        for (int i = 0; i < n; ++i) cap_e[i] = d.asymptote[i] - dist;
        const double max_span = task_span >= 0.0 ? task_span : span_of(d);
        int32_t n_trial = 1024;
        if (alg.integration_step > 0) {
            const double want = std::ceil(max_span / to_hartree(alg.integration_step));
            n_trial = (int32_t)std::min(std::max(want, 64.0), (double)(1 << 22));
        }
        epscu_batch b{n, d.V.data(), d.offsets.data(), d.N.data(), d.r_min.data(), d.r_max.data(), mus.data(),
                      cap_e.data(), n_trial, (int32_t)alg.min_level, (int32_t)alg.max_level};
        std::vector<int32_t> n_total(n), n_out(n), nodes((size_t)n * cap), status((size_t)n * cap);
        std::vector<double> energy((size_t)n * cap), err((size_t)n * cap);
        std::vector<int64_t> psi_off(n);
        std::vector<double> psi;
        if (cfg.want_wavefunctions) {
            int64_t pts = 0;
            for (int i = 0; i < n; ++i) pts += d.N[i];
            psi.assign((size_t)(pts * cap), 0.0);
        }
        epscu_result r{cap, n_total.data(), n_out.data(), energy.data(), nodes.data(), status.data(), err.data(),
                       psi.empty() ? nullptr : psi.data(), (int64_t)psi.size(), psi_off.data(), 0};
        epscu_opts o{};
        o.method = method;
        o.flags = psi.empty() ? 0 : EPSCU_WANT_PSI;
        o.tol = 1e-12;
        setMessage("solving potentials " + std::to_string(first) + ".." + std::to_string(first + count));
        epscu_status s;
        {
            std::lock_guard<std::mutex> solve_guard(device->solveMutex());
            {
                std::lock_guard<std::mutex> g(run_mu);
                if (st.stop_requested()) {
                    setMessage("cancelled");
                    return;
                }
                in_solve = true;
            }
            s = epscu_solve(ctx, &b, &r, &o);
            std::lock_guard<std::mutex> g(run_mu);
            in_solve = false;
            // a request that reached the context after the solve consumed its
            // flag would stop the next solve of another task: withdraw it
            if (st.stop_requested()) epscu_cancel_clear(ctx);
        }
        if (s == EPSCU_ERR_CANCELLED || st.stop_requested()) {
            setMessage("cancelled");
            return;
        }
        check("epscu_solve", s);
        const double psi_scale = 1.0 / std::sqrt(kBohrAngstrom);  // bohr^-1/2 -> angstrom^-1/2
        for (int i = 0; i < n; ++i) {
            const int k = n_out[i];
            res.n_total.push_back(n_total[i]);
            res.N.push_back(d.N[i]);
            res.r_min.push_back(d.r_min[i] * kBohrAngstrom);
            res.r_max.push_back(d.r_max[i] * kBohrAngstrom);
            std::vector<double> e(k), ee(k);
            std::vector<int32_t> nd(k), stt(k);
            for (int s2 = 0; s2 < k; ++s2) {
                const size_t q = (size_t)i * cap + s2;
                e[s2] = energy[q] * kHartreeInvCm;
                ee[s2] = err[q] * kHartreeInvCm;
                nd[s2] = nodes[q];
                stt[s2] = status[q];
            }
            res.energies.push_back(std::move(e));
            res.error_estimate.push_back(std::move(ee));
            res.nodes.push_back(std::move(nd));
            res.status.push_back(std::move(stt));
            if (!psi.empty()) {
                std::vector<double> w((size_t)k * d.N[i]);
                for (size_t j = 0; j < w.size(); ++j) w[j] = psi[(size_t)psi_off[i] + j] * psi_scale;
                res.wavefunctions.push_back(std::move(w));
            } else {
                res.wavefunctions.emplace_back();
            }
        }
    }
    int64_t levels = 0;
    for (auto& e : res.energies) levels += (int64_t)e.size();
    setMessage("done: " + std::to_string(levels) + " levels from " + std::to_string(total) + " potentials");
}

template class TaskHandle<float>;
template class TaskHandle<double>;

}  // namespace epseon::cuda::cpp
