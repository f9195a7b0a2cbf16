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

// Nodal charge density [C/m^3], index = node (NodeChargeDensitiesMap).
using NodeChargeDensities = std::vector<double>;

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

    spg_handle *handle() { return h_; }
    int64_t n_nodes() const { return n_nodes_; }
    int64_t n_tets() const { return n_tets_; }
    int64_t n_triangles() const { return n_triangles_; }
    int64_t n_particles() const { return n_particles_; }

    void set_particles(const std::vector<double> &pos, const std::vector<double> &vel) {
        if (pos.size() != vel.size() || pos.size() % 3) throw PICBaseException("pos/vel size mismatch", -1);
        n_particles_ = int64_t(pos.size() / 3);
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
        check(spg_run(h_, nsteps, &st));
        return st;
    }
    template <class E = PICBaseException>
    void check(int rc) {
        if (rc != SPG_OK) throw E(spg_last_error(h_), rc);
    }

private:
    spg_handle *h_ = nullptr;
    int64_t n_nodes_ = 0, n_tets_ = 0, n_triangles_ = 0, n_particles_ = 0;
};

class NodeChargeDensityProcessor {
public:
    // Deposits every non-settled particle and returns nodal charge density.
    static void gather(double /*timeMoment*/, ParticleInCellEngine &engine, NodeChargeDensities &out) {
        out.resize(size_t(engine.n_nodes()));
        engine.check<PICNodeChargeDensityProcessorOmpVersionHelperException>(
            spg_gather(engine.handle(), out.data()));
    }
};

class ChargeDensityEquationSolver {
public:
    // Poisson solve from the nodal charge density, then E per tet.
    static void solve(double /*timeMoment*/, const NodeChargeDensities &rho, ParticleInCellEngine &engine,
                      std::vector<double> *potential_out = nullptr, int32_t *iterations = nullptr) {
        if (rho.size() != size_t(engine.n_nodes()))
            throw PICChargeDensityEquationSolverSolvingException("rho has the wrong size", SPG_E_INVALID);
        std::vector<double> phi;
        if (potential_out) potential_out->resize(size_t(engine.n_nodes()));
        int32_t it = 0;
        double rr = 0.0;
        engine.check<PICChargeDensityEquationSolverSolvingException>(spg_solve(
            engine.handle(), rho.data(), potential_out ? potential_out->data() : nullptr, &it, &rr));
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
