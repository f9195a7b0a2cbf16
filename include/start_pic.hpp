// start_pic.hpp -- C++ host interface with the reference's ParticleInCellEngine
// names, over the C ABI of libstart_gpu.so (start_gpu.h). Header-only.
//
// Reference surface kept (static methods, same call order in the time loop):
//   NodeChargeDensityProcessor::gather
//     include/ParticleInCellEngine/NodeChargeDensityProcessor.hpp:39-46
//   ChargeDensityEquationSolver::solve
//     include/ParticleInCellEngine/ChargeDensityEquationSolver.hpp:38-42
//   ParticleDynamicsProcessor::process
//     include/ParticleInCellEngine/ParticleDynamicsProcessor/ParticleDynamicsProcessor.hpp:154-170
// Errors surface as the reference's exception types
// (include/ParticleInCellEngine/PICExceptions.hpp). The heavyweight reference
// arguments (CubicGrid, GSMAssembler, SurfaceMesh, tracker maps, mutexes) are
// all state that the engine handle owns on the GPU, so they collapse into one
// ParticleInCellEngine reference.
#pragma once

#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "start_gpu.h"

namespace start {

struct PICBaseException : std::runtime_error {
    int code;
    PICBaseException(const std::string &m, int c) : std::runtime_error(m), code(c) {}
};
struct PICUnknownException : PICBaseException {
    using PICBaseException::PICBaseException;
};
struct PICNodeChargeDensityProcessorOmpVersionHelperException : PICBaseException {
    using PICBaseException::PICBaseException;
};
struct PICChargeDensityEquationSolverSolvingException : PICBaseException {
    using PICBaseException::PICBaseException;
};
struct PICParticleDynamicsProcessorProcessingException : PICBaseException {
    using PICBaseException::PICBaseException;
};

// Tet mesh in SI units; node index = gmsh tag - 1.
struct Mesh {
    std::vector<double> nodes;         // 3 per node
    std::vector<int32_t> tets;         // 4 per tet
    std::vector<int32_t> triangles;    // 3 per surface triangle; id = row
    std::map<int32_t, double> boundary_conditions;  // node -> volts (BoundaryConditionsMap)
};

class ParticleInCellEngine;

// Nodal charge density [C/m^3], index = node: the NodeChargeDensitiesMap that
// NodeChargeDensityProcessor::gather fills and ChargeDensityEquationSolver::
// solve reads (include/ParticleInCellEngine/PICTypes.hpp).
//
// After gather the values stay on the GPU. The first read (operator[],
// data(), values()) copies them down with spg_get_charge_density; a solve of
// a density nobody wrote to since its gather uses the device copy and moves
// nothing through the host. Writing through a non-const accessor, or
// assign(), makes the host values the ones the next solve uploads. A density
// that is still on the device must be read while its engine is alive and
// before the engine's charge changes again (the next gather, a solve of
// another density, a run, new particles); a later read throws
// PICNodeChargeDensityProcessorOmpVersionHelperException.
class NodeChargeDensities {
public:
    NodeChargeDensities() = default;
    explicit NodeChargeDensities(std::vector<double> v) { assign(std::move(v)); }

    size_t size() const { return n_; }
    bool empty() const { return n_ == 0; }
    double operator[](size_t i) const { return host()[i]; }
    double &operator[](size_t i) { return writable()[i]; }
    const double *data() const { return host().data(); }
    double *data() { return writable().data(); }
    const std::vector<double> &values() const { return host(); }
    std::vector<double> &values() { return writable(); }
    void assign(std::vector<double> v) {
        vals_ = std::move(v);
        n_ = vals_.size();
        state_ = kHost;
        eng_ = nullptr;
    }
    // true while the values live only on the GPU (no host copy taken yet)
    bool on_device_only() const { return state_ == kDevice; }

private:
    friend class NodeChargeDensityProcessor;
    friend class ChargeDensityEquationSolver;
    enum State { kHost, kDevice, kSynced };

    const std::vector<double> &host() const;
    std::vector<double> &writable() {
        host();
        state_ = kHost;
        return vals_;
    }

    mutable std::vector<double> vals_;
    mutable State state_ = kHost;
    size_t n_ = 0;
    const ParticleInCellEngine *eng_ = nullptr;
    uint64_t generation_ = 0;
};

struct Particles {
    std::vector<double> pos, vel;  // 3 per particle, SI
    std::vector<int32_t> tet;
    std::vector<uint32_t> flags;   // SPG_FLAG_SETTLED / SPG_FLAG_LOST
};

class ParticleInCellEngine {
public:
    ParticleInCellEngine(const Mesh &mesh, const spg_params &params) {
        std::vector<int32_t> dn;
        std::vector<double> dv;
        for (const auto &kv : mesh.boundary_conditions) {
            dn.push_back(kv.first);
            dv.push_back(kv.second);
        }
        spg_mesh_desc d{};
        d.n_nodes = int64_t(mesh.nodes.size() / 3);
        d.node_xyz = mesh.nodes.data();
        d.n_tets = int64_t(mesh.tets.size() / 4);
        d.tet_nodes = mesh.tets.data();
        d.n_triangles = int64_t(mesh.triangles.size() / 3);
        d.tri_nodes = mesh.triangles.data();
        d.n_dirichlet = int64_t(dn.size());
        d.dirichlet_nodes = dn.data();
        d.dirichlet_values = dv.data();
        const int rc = spg_create(&d, &params, &h_);
        if (rc != SPG_OK) throw PICBaseException(spg_last_error(nullptr), rc);
        int64_t info[6];
        spg_mesh_info(h_, info);
        n_nodes_ = info[0];
        n_tets_ = info[1];
        n_triangles_ = info[2];
    }
    ~ParticleInCellEngine() { spg_destroy(h_); }
    ParticleInCellEngine(const ParticleInCellEngine &) = delete;
    ParticleInCellEngine &operator=(const ParticleInCellEngine &) = delete;

    spg_handle *handle() const { return h_; }
    int64_t n_nodes() const { return n_nodes_; }
    int64_t n_tets() const { return n_tets_; }
    int64_t n_triangles() const { return n_triangles_; }
    int64_t n_particles() const { return n_particles_; }

    void set_particles(const std::vector<double> &pos, const std::vector<double> &vel) {
        if (pos.size() != vel.size() || pos.size() % 3) throw PICBaseException("pos/vel size mismatch", -1);
        n_particles_ = int64_t(pos.size() / 3);
        next_charge_generation();
        check(spg_set_particles(h_, n_particles_, pos.data(), vel.data(), nullptr));
    }
    Particles particles() {
        Particles p;
        p.pos.resize(3 * n_particles_);
        p.vel.resize(3 * n_particles_);
        p.tet.resize(n_particles_);
        p.flags.resize(n_particles_);
        check(spg_get_particles(h_, n_particles_, p.pos.data(), p.vel.data(), p.tet.data(), p.flags.data()));
        return p;
    }
    std::vector<uint64_t> triangle_counts() {
        std::vector<uint64_t> c(n_triangles_);
        check(spg_get_triangle_counts(h_, c.data()));
        return c;
    }
    spg_stats run(int32_t nsteps) {
        spg_stats st{};
        next_charge_generation();
        check(spg_run(h_, nsteps, &st));
        return st;
    }
    template <class E = PICBaseException>
    void check(int rc) {
        if (rc != SPG_OK) throw E(spg_last_error(h_), rc);
    }
    // Changes each time the handle's nodal charge may have changed (a deposit,
    // a solve of a given density, a run, new particles).
    uint64_t charge_generation() const { return charge_generation_; }
    uint64_t next_charge_generation() { return ++charge_generation_; }

private:
    spg_handle *h_ = nullptr;
    int64_t n_nodes_ = 0, n_tets_ = 0, n_triangles_ = 0, n_particles_ = 0;
    uint64_t charge_generation_ = 0;
};

inline const std::vector<double> &NodeChargeDensities::host() const {
    if (state_ == kDevice) {
        if (eng_->charge_generation() != generation_)
            throw PICNodeChargeDensityProcessorOmpVersionHelperException(
                "nodal charge density read after the engine's charge changed", SPG_E_STATE);
        vals_.resize(n_);
        const int rc = spg_get_charge_density(eng_->handle(), vals_.data());
        if (rc != SPG_OK)
            throw PICNodeChargeDensityProcessorOmpVersionHelperException(spg_last_error(eng_->handle()), rc);
        state_ = kSynced;
    }
    return vals_;
}

class NodeChargeDensityProcessor {
public:
    // Deposits every non-settled particle; `out` refers to the density the
    // deposit left on the GPU (read on first access).
    static void gather(double /*timeMoment*/, ParticleInCellEngine &engine, NodeChargeDensities &out) {
        engine.check<PICNodeChargeDensityProcessorOmpVersionHelperException>(spg_gather(engine.handle(), nullptr));
        out.n_ = size_t(engine.n_nodes());
        out.state_ = NodeChargeDensities::kDevice;
        out.eng_ = &engine;
        out.generation_ = engine.next_charge_generation();
    }
};

class ChargeDensityEquationSolver {
public:
    // Poisson solve from the nodal charge density, then E per tet. A density
    // that came from this engine's latest gather and was not written to is
    // solved from the device copy; any other is uploaded.
    static void solve(double /*timeMoment*/, const NodeChargeDensities &rho, ParticleInCellEngine &engine,
                      std::vector<double> *potential_out = nullptr, int32_t *iterations = nullptr) {
        if (rho.size() != size_t(engine.n_nodes()))
            throw PICChargeDensityEquationSolverSolvingException("rho has the wrong size", SPG_E_INVALID);
        const bool resident = rho.eng_ == &engine && rho.generation_ == engine.charge_generation() &&
                              rho.state_ != NodeChargeDensities::kHost;
        const double *up = resident ? nullptr : rho.data();
        if (!resident) engine.next_charge_generation();
        if (potential_out) potential_out->resize(size_t(engine.n_nodes()));
        int32_t it = 0;
        double rr = 0.0;
        engine.check<PICChargeDensityEquationSolverSolvingException>(
            spg_solve(engine.handle(), up, potential_out ? potential_out->data() : nullptr, &it, &rr));
        if (iterations) *iterations = it;
    }
};

class ParticleDynamicsProcessor {
public:
    // One step of push, move, gas collision and surface settle for every particle.
    static spg_stats process(ParticleInCellEngine &engine, double /*timeMoment*/, int32_t nsteps = 1) {
        spg_stats st{};
        engine.check<PICParticleDynamicsProcessorProcessingException>(spg_process(engine.handle(), nsteps, &st));
        return st;
    }
};

}  // namespace start
