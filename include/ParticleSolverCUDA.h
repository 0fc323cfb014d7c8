// ParticleSolverCUDA -- a drop-in ParticleSolver (MarcVivas/N-body,
// include/ParticleSolver.h:8-15) backed by the sm_103a solver in
// libnbody_gb300 through its C ABI (nbody_gb300.h).
//
// Mode::DirectSum replaces ParticleSolverCPUParallel (-v 2; GPU form -v 3/-v 4),
// Mode::BarnesHut replaces ParticleSolverBHutCPUParallel (-v 6; GPU form -v 7).
// Construction mirrors theirs: (timeStep, squaredSoftening[, n]) plus the mode,
// the squared opening angle (the reference hard-codes 0.25,
// src/Octree/Octree.cpp:15) and the CUDA device.
//
// updateParticlePositions keeps the reference's contract for solvers whose
// usesGPU() is false: positions, velocities, accelerations and forces of the
// ParticleSystem are valid host arrays after every call (they are copied to
// the GPU, advanced one step, and copied back), so ParticleSimulation and
// ParticleDrawer need no change. Errors throw std::runtime_error, as the
// reference's Shader does for a missing file.
//
// Header-only; needs the reference's include/ directory on the include path
// and links against libnbody_gb300.so.
#ifndef NBODY_GB300_PARTICLE_SOLVER_CUDA_H
#define NBODY_GB300_PARTICLE_SOLVER_CUDA_H

#include <stdexcept>
#include <string>

#include "ParticleSolver.h"
#include "ParticleSystem.h"
#include "nbody_gb300.h"

class ParticleSolverCUDA : public ParticleSolver {
public:
    enum class Mode { DirectSum = NBODY_MODE_PP, BarnesHut = NBODY_MODE_BH };

    ParticleSolverCUDA(float timeStep, float squaredSoftening, int n, Mode mode, float theta2 = 0.25f,
                       int device = 0)
        : n_(static_cast<unsigned int>(n)) {
        static_assert(sizeof(glm::vec4) == 4 * sizeof(float), "ParticleSystem vec4 must be four packed floats");
        const int rc = nbody_create(&ctx_, device, static_cast<int>(mode), n, timeStep, squaredSoftening, theta2);
        if (rc != NBODY_OK) throw std::runtime_error(std::string("ParticleSolverCUDA: ") + nbody_status_string(rc));
    }

    ParticleSolverCUDA(const ParticleSolverCUDA &) = delete;
    ParticleSolverCUDA &operator=(const ParticleSolverCUDA &) = delete;

    ~ParticleSolverCUDA() override {
        if (ctx_) nbody_destroy(ctx_);
    }

    // One step: forces at the current positions, then the reference integrator
    // (include/ParticleSystem.h:52-69); forces[] receives the new acceleration.
    void updateParticlePositions(ParticleSystem *particles) override {
        if (!particles || particles->size() != n_)
            throw std::runtime_error("ParticleSolverCUDA: system size differs from the solver's");
        const int rc = nbody_update_host(ctx_, reinterpret_cast<float *>(particles->getPositions()),
                                         reinterpret_cast<float *>(particles->getVelocities()),
                                         reinterpret_cast<float *>(particles->getAccelerations()),
                                         reinterpret_cast<const float *>(particles->getMasses()),
                                         reinterpret_cast<float *>(particles->getForces()), 1);
        if (rc != NBODY_OK)
            throw std::runtime_error(std::string("ParticleSolverCUDA: ") + nbody_status_string(rc) + " " +
                                     nbody_last_error(ctx_));
    }

    float getSquaredSoftening() override { return nbody_get_squared_softening(ctx_); }

    // Host arrays stay valid after every call (see above).
    bool usesGPU() override { return false; }

    nbody_ctx *context() { return ctx_; }

private:
    nbody_ctx *ctx_ = nullptr;
    unsigned int n_;
};

#endif  // NBODY_GB300_PARTICLE_SOLVER_CUDA_H
