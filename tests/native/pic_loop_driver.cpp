// The time loop of ModelingMainDriver::startModeling (src/ModelingMainDriver.cpp:146-184)
// written against include/start_pic.hpp the way a Start maintainer would call it:
//
//   NodeChargeDensityProcessor::gather -> ChargeDensityEquationSolver::solve
//   -> ParticleDynamicsProcessor::process, stopping once no particle is alive.
//
// Input (binary, little-endian, written by the GPU test):
//   "SPGLOOP1", int64 sizeof(spg_params), spg_params bytes,
//   int64 n_nodes, f64 nodes[3 n_nodes], int64 n_tets, i32 tets[4 n_tets],
//   int64 n_tris, i32 tris[3 n_tris], int64 n_dir, i32 dir_nodes[n_dir],
//   f64 dir_values[n_dir], int64 n_particles, f64 pos[3 n], f64 vel[3 n],
//   int64 steps, int64 solve_every
// Output (binary): int64 steps_run, int64 n_alive, int64 cg_iters_last,
//   f64 pos[3 n], f64 vel[3 n], i32 tet[n], u32 flags[n], u64 counts[n_tris],
//   f64 rho[n_nodes] of the last gather (read lazily through NodeChargeDensities),
//   f64 phi[n_nodes] of the last loop solve,
//   f64 phi_res[n_nodes]: that density solved again from its device copy,
//   f64 phi_up[n_nodes]: solved again after a host round trip (uploaded),
//   int64 resident_before_read (1 if the last gather's density was still GPU-only).
// Exit status 0 on success; a thrown PICBaseException prints its message and code.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "start_pic.hpp"

namespace {

struct Reader {
    std::ifstream f;
    explicit Reader(const char *path) : f(path, std::ios::binary) {
        if (!f) throw std::runtime_error(std::string("cannot open ") + path);
    }
    template <class T>
    T get() {
        T v;
        f.read(reinterpret_cast<char *>(&v), sizeof(T));
        if (!f) throw std::runtime_error("input truncated");
        return v;
    }
    template <class T>
    std::vector<T> vec(size_t n) {
        std::vector<T> v(n);
        f.read(reinterpret_cast<char *>(v.data()), std::streamsize(n * sizeof(T)));
        if (!f) throw std::runtime_error("input truncated");
        return v;
    }
};

template <class T>
void put(std::ofstream &o, const T &v) {
    o.write(reinterpret_cast<const char *>(&v), sizeof(T));
}
template <class T>
void put(std::ofstream &o, const std::vector<T> &v) {
    o.write(reinterpret_cast<const char *>(v.data()), std::streamsize(v.size() * sizeof(T)));
}

}  // namespace

int main(int argc, char **argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s input.bin output.bin\n", argv[0]);
        return 2;
    }
    try {
        Reader in(argv[1]);
        char magic[8];
        in.f.read(magic, 8);
        if (!in.f || std::memcmp(magic, "SPGLOOP1", 8) != 0) throw std::runtime_error("bad input magic");
        if (in.get<int64_t>() != int64_t(sizeof(spg_params))) throw std::runtime_error("spg_params size differs");
        const spg_params prm = in.get<spg_params>();

        start::Mesh mesh;
        const int64_t nn = in.get<int64_t>();
        mesh.nodes = in.vec<double>(size_t(3 * nn));
        const int64_t nt = in.get<int64_t>();
        mesh.tets = in.vec<int32_t>(size_t(4 * nt));
        const int64_t ntri = in.get<int64_t>();
        mesh.triangles = in.vec<int32_t>(size_t(3 * ntri));
        const int64_t nd = in.get<int64_t>();
        const std::vector<int32_t> dn = in.vec<int32_t>(size_t(nd));
        const std::vector<double> dv = in.vec<double>(size_t(nd));
        for (int64_t k = 0; k < nd; ++k) mesh.boundary_conditions[dn[k]] = dv[k];
        const int64_t np = in.get<int64_t>();
        const std::vector<double> pos = in.vec<double>(size_t(3 * np));
        const std::vector<double> vel = in.vec<double>(size_t(3 * np));
        const int64_t steps = in.get<int64_t>();
        const int64_t solve_every = in.get<int64_t>();

        // --- once, after FEM initialisation
        start::ParticleInCellEngine engine(mesh, prm);
        engine.set_particles(pos, vel);

        // --- the time loop
        start::NodeChargeDensities rho;
        std::vector<double> phi;
        int32_t iters = 0;
        int64_t k = 0;
        const double dt = prm.dt;
        for (; k < steps; ++k) {
            const double t = double(k) * dt;
            if (k % solve_every == 0) {
                start::NodeChargeDensityProcessor::gather(t, engine, rho);
                start::ChargeDensityEquationSolver::solve(t, rho, engine, &phi, &iters);
            }
            const spg_stats st = start::ParticleDynamicsProcessor::process(engine, t);
            if (st.n_alive == 0) {
                ++k;
                break;  // StopSubject: every particle has settled
            }
        }
        const int64_t resident = rho.on_device_only() ? 1 : 0;

        // --- finalisation
        const start::Particles p = engine.particles();
        const std::vector<uint64_t> counts = engine.triangle_counts();
        std::vector<double> rho_host = rho.values();  // lazy download of the last gather

        // the last density solved twice more, warm started from the loop's
        // potential: from its device copy, then as host values (uploaded)
        std::vector<double> phi_res, phi_up;
        start::ChargeDensityEquationSolver::solve(0.0, rho, engine, &phi_res);
        start::NodeChargeDensities copy(rho_host);
        start::ChargeDensityEquationSolver::solve(0.0, copy, engine, &phi_up);
        spg_stats st{};
        engine.check(spg_get_stats(engine.handle(), &st));

        std::ofstream out(argv[2], std::ios::binary);
        put(out, k);
        put(out, st.n_alive);
        put(out, int64_t(iters));
        put(out, p.pos);
        put(out, p.vel);
        put(out, p.tet);
        put(out, p.flags);
        put(out, counts);
        put(out, rho_host);
        put(out, phi);
        put(out, phi_res);
        put(out, phi_up);
        put(out, resident);
        if (!out) throw std::runtime_error("cannot write output");
    } catch (const start::PICBaseException &e) {
        std::fprintf(stderr, "PICBaseException (code %d): %s\n", e.code, e.what());
        return 1;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
