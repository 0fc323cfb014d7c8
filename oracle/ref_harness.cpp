// C-ABI harness around the reference's own CPU solvers, compiled unmodified
// from the reference sources together with the headless shim (oracle/shim).
// Test infrastructure only: it is the parity oracle and the CPU baseline, never
// the product. It builds a ParticleSystem from the caller's arrays the way the
// reference's initialisers do (Particle(pos, vel, acc, mass), then
// ParticleSystem(particles, usesGPU=false); include/ParticleSystem.h:33,
// src/ParticleSystem/ParticleSystem.cpp:5-24), then calls
// ParticleSolver::updateParticlePositions (include/ParticleSolver.h:12) `steps`
// times, timing only that call with steady_clock.
#include <omp.h>

#include <chrono>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "Octree.h"
#include "ParallelOctreeCPU.h"
#include "Particle.h"
#include "ParticleSolver.h"
#include "ParticleSolverBHutCPUParallel.h"
#include "ParticleSolverBHutCPUSeq.h"
#include "ParticleSolverCPUParallel.h"
#include "ParticleSolverCPUSequential.h"
#include "ParticleSystem.h"
#include "ParticleSystemFile.h"
#include "ParticleSystemLagrange.h"

namespace {

// Exposes the protected octree of the BH solvers so that the opening angle
// (public member Octree::theta, include/Octree.h:18) can be set and the root
// mass read back after a step.
struct BHParallel : ParticleSolverBHutCPUParallel {
    using ParticleSolverBHutCPUParallel::ParticleSolverBHutCPUParallel;
    Octree *tree() { return octree; }
};
struct BHSeq : ParticleSolverBHutCPUSeq {
    using ParticleSolverBHutCPUSeq::ParticleSolverBHutCPUSeq;
    Octree *tree() { return octree; }
};

std::unique_ptr<ParticleSystem> make_system(int n, const float *pos4, const float *vel4,
                                            const float *acc4, const float *mass) {
    std::vector<Particle> ps;
    ps.reserve(n);
    for (int i = 0; i < n; ++i) {
        glm::vec3 p(pos4[4 * i], pos4[4 * i + 1], pos4[4 * i + 2]);
        glm::vec3 v(vel4[4 * i], vel4[4 * i + 1], vel4[4 * i + 2]);
        glm::vec3 a(acc4 ? acc4[4 * i] : 0.f, acc4 ? acc4[4 * i + 1] : 0.f, acc4 ? acc4[4 * i + 2] : 0.f);
        ps.emplace_back(p, v, a, mass[i]);
    }
    return std::make_unique<ParticleSystem>(ps, false);
}

void read_back(ParticleSystem &sys, int n, float *pos4, float *vel4, float *acc4, float *force4) {
    for (int i = 0; i < n; ++i) {
        const glm::vec4 &p = sys.getPositions()[i];
        const glm::vec4 &v = sys.getVelocities()[i];
        const glm::vec4 &a = sys.getAccelerations()[i];
        const glm::vec4 &f = sys.getForces()[i];
        if (pos4) { pos4[4 * i] = p.x; pos4[4 * i + 1] = p.y; pos4[4 * i + 2] = p.z; pos4[4 * i + 3] = p.w; }
        if (vel4) { vel4[4 * i] = v.x; vel4[4 * i + 1] = v.y; vel4[4 * i + 2] = v.z; vel4[4 * i + 3] = v.w; }
        if (acc4) { acc4[4 * i] = a.x; acc4[4 * i + 1] = a.y; acc4[4 * i + 2] = a.z; acc4[4 * i + 3] = a.w; }
        if (force4) { force4[4 * i] = f.x; force4[4 * i + 1] = f.y; force4[4 * i + 2] = f.z; force4[4 * i + 3] = f.w; }
    }
}

}  // namespace

extern "C" {

// version: 1 = ParticleSolverCPUSequential (-v 1), 2 = ParticleSolverCPUParallel (-v 2),
//          5 = ParticleSolverBHutCPUSeq (-v 5),   6 = ParticleSolverBHutCPUParallel (-v 6).
// theta2 <= 0 keeps the reference's hard-coded 0.25 (src/Octree/Octree.cpp:15).
// threads <= 0 keeps OpenMP's default. Returns 0 on success, -1 on a bad version.
int ref_run(int version, int n, const float *pos4, const float *vel4, const float *acc4,
            const float *mass, float dt, float eps2, float theta2, int steps, int threads,
            float *pos4_out, float *vel4_out, float *acc4_out, float *force4_out,
            double *seconds_out, float *root_mass_out) {
    if (threads > 0) omp_set_num_threads(threads);
    auto sys = make_system(n, pos4, vel4, acc4, mass);
    std::unique_ptr<ParticleSolver> solver;
    Octree *tree = nullptr;
    switch (version) {
        case 1: solver = std::make_unique<ParticleSolverCPUSequential>(dt, eps2); break;
        case 2: solver = std::make_unique<ParticleSolverCPUParallel>(dt, eps2); break;
        case 5: { auto s = std::make_unique<BHSeq>(dt, eps2, n); tree = s->tree(); solver = std::move(s); break; }
        case 6: { auto s = std::make_unique<BHParallel>(dt, eps2, n); tree = s->tree(); solver = std::move(s); break; }
        default: return -1;
    }
    if (tree && theta2 > 0.f) tree->theta = theta2;
    double secs = 0.0;
    for (int s = 0; s < steps; ++s) {
        auto t0 = std::chrono::steady_clock::now();
        solver->updateParticlePositions(sys.get());
        auto t1 = std::chrono::steady_clock::now();
        secs += std::chrono::duration<double>(t1 - t0).count();
    }
    if (seconds_out) *seconds_out = secs;
    if (root_mass_out) *root_mass_out = tree ? tree->getNodes()[0].getMass() : 0.f;
    read_back(*sys, n, pos4_out, vel4_out, acc4_out, force4_out);
    return 0;
}

// The reference's one deterministic initialiser (-i 3,
// src/ParticleSystemInitializer/ParticleSystemLagrange/ParticleSystemLagrange.cpp:8-50):
// three equal masses on an equilateral triangle. Writes 3 bodies.
int ref_lagrange(float wx, float wy, float wz, float *pos4, float *vel4, float *acc4, float *mass) {
    ParticleSystemLagrange init;
    auto sys = init.generateParticles(glm::vec3(wx, wy, wz), false);
    read_back(*sys, 3, pos4, vel4, acc4, nullptr);
    for (int i = 0; i < 3; ++i) mass[i] = sys->getMasses()[i].x;
    return 3;
}

// Text dump of a system with the reference's writer
// (src/ParticleSystem/ParticleSystem.cpp:205-215). Returns the byte count
// written into `out` (truncated at cap), or the needed size when out is NULL.
long ref_dump_text(int n, const float *pos4, const float *vel4, const float *acc4,
                   const float *mass, char *out, long cap) {
    auto sys = make_system(n, pos4, vel4, acc4, mass);
    std::ostringstream os;
    os << *sys;
    const std::string s = os.str();
    if (!out) return static_cast<long>(s.size());
    long m = static_cast<long>(s.size()) < cap ? static_cast<long>(s.size()) : cap;
    std::memcpy(out, s.data(), static_cast<size_t>(m));
    return m;
}

// Loads a text dump with the reference's reader (-f,
// src/ParticleSystemInitializer/ParticleSystemFile/ParticleSystemFile.cpp:10-90).
// Returns the body count, writing at most cap bodies.
int ref_load_text(const char *path, int cap, float *pos4, float *vel4, float *acc4, float *mass) {
    ParticleSystemFile init{std::string(path)};
    auto sys = init.generateParticles(glm::vec3(0.f), false);
    int n = static_cast<int>(sys->size());
    int m = n < cap ? n : cap;
    std::vector<float> p(4 * n), v(4 * n), a(4 * n);
    read_back(*sys, n, p.data(), v.data(), a.data(), nullptr);
    std::memcpy(pos4, p.data(), sizeof(float) * 4 * m);
    std::memcpy(vel4, v.data(), sizeof(float) * 4 * m);
    std::memcpy(acc4, a.data(), sizeof(float) * 4 * m);
    for (int i = 0; i < m; ++i) mass[i] = sys->getMasses()[i].x;
    return n;
}

// Builds one -v 6 tree (ParallelOctreeCPU::reset + insert,
// src/Octree/ParallelOctreeCPU.cpp:76-206) and copies out up to `cap` nodes as
// 12 floats each: mass, firstChild, next, com.xyz, min.xyz, max.xyz. Returns the
// node-pool size (ParallelOctreeCPU::getMaxNodes).
long ref_bh_tree(int n, const float *pos4, const float *mass, float *out, long cap) {
    std::vector<float> zero(4 * static_cast<size_t>(n), 0.f);
    auto sys = make_system(n, pos4, zero.data(), zero.data(), mass);
    ParallelOctreeCPU tree(n);
    tree.reset(sys.get());
    tree.insert(sys.get());
    const long total = tree.getMaxNodes();
    const long m = total < cap ? total : cap;
    const Node *nodes = tree.getNodes();
    for (long i = 0; i < m; ++i) {
        const Node &d = nodes[i];
        float *o = out + 12 * i;
        o[0] = d.getMass(); o[1] = static_cast<float>(d.getFirstChild()); o[2] = static_cast<float>(d.getNext());
        const glm::vec4 c = d.getCenterOfMass(), lo = d.getMinBoundary(), hi = d.getMaxBoundary();
        o[3] = c.x; o[4] = c.y; o[5] = c.z; o[6] = lo.x; o[7] = lo.y; o[8] = lo.z; o[9] = hi.x; o[10] = hi.y; o[11] = hi.z;
    }
    return total;
}

}  // extern "C"
