/* nbody_gb300 — C ABI of the GB300-native (sm_103a) gravity solve.
 *
 * This is the drop-in boundary for the reference's solver plugin interface,
 * MarcVivas/N-body `class ParticleSolver` (include/ParticleSolver.h:8-15):
 *   updateParticlePositions(ParticleSystem*)   -> nbody_update_host
 *   getSquaredSoftening()                       -> nbody_get_squared_softening
 *   usesGPU()                                   -> (host arrays stay valid after
 *                                                   every call: the adapter in
 *                                                   ParticleSolverCUDA.h returns false)
 * and for the solver constructors it replaces:
 *   ParticleSolverCPUParallel(float timeStep, float squaredSoftening)
 *     (include/ParticleSolverCPUParallel.h:9, -v 2; GPU form -v 3/-v 4,
 *      include/ParticleSolverGPU.h)                    -> nbody_create(.., NBODY_MODE_PP, ..)
 *   ParticleSolverBHutCPUParallel(float timeStep, float squaredSoftening, int n)
 *     (include/ParticleSolverBHutCPUParallel.h:9, -v 6; GPU form -v 7)
 *                                                       -> nbody_create(.., NBODY_MODE_BH, ..)
 *
 * Plain pointers and sizes only. Every entry point returns an int status
 * (NBODY_OK or an NBODY_ERR_* code); no exception crosses this boundary. A
 * context is not re-entrant: calls on one context must not overlap.
 *
 * Host arrays use the reference's ParticleSystem layout
 * (include/ParticleSystem.h:100-104): float[4*n] per quantity, one (x,y,z,w)
 * vec4 per body; positions carry w = 0 and masses live in masses4[4*i].
 * Device-resident state uses this library's layout: pos_mass float4
 * (x, y, z, m), vel float4 (x, y, z, 0), acc float4 (x, y, z, 0).
 */
#ifndef NBODY_GB300_H
#define NBODY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NBODY_OK 0
#define NBODY_ERR_ARG 1      /* bad argument (null pointer, n <= 0, unknown mode, ...) */
#define NBODY_ERR_CUDA 2     /* a CUDA runtime call failed (see nbody_last_error)      */
#define NBODY_ERR_NOMEM 3    /* device or pinned allocation failed                     */
#define NBODY_ERR_CAPACITY 4 /* a fixed-size device structure would overflow           */
#define NBODY_ERR_TIMEOUT 5  /* a bounded device-side wait gave up                     */
#define NBODY_ERR_STATE 6    /* call out of order (e.g. step before upload)            */

#define NBODY_MODE_PP 0 /* direct sum, reference -v 2 (CPU) / -v 3, -v 4 (GLSL)   */
#define NBODY_MODE_BH 1 /* Barnes-Hut, reference -v 6 (CPU) / -v 7 (GLSL)         */

/* 63-bit keys that order bodies for the Barnes-Hut tree (21 bits per axis,
 * x highest in each bit triple, over the per-step root box):
 * NBODY_KEYS_OCTREE (default): the reference's own octree descent taken 21
 *   levels deep -- per level and axis centre = min + (max - min) / 2 in FP32,
 *   upper half unless pos < centre (Octree::getNextNode / Octree::subdivide,
 *   src/Octree/Octree.cpp:148-231). Cells are then exactly the reference's.
 * NBODY_KEYS_MORTON: the reference's GLSL Morton quantisation extended to 21
 *   bits, q = uint(clamp((p - min) / max(max - min, 1e-6) * 2^21, 0, 2^21 - 1))
 *   (src/shaders/ComputeShaders/morton.glsl:37-75). The two differ only for
 *   bodies within rounding of a cell boundary. */
#define NBODY_KEYS_OCTREE 0
#define NBODY_KEYS_MORTON 1

/* Integrator applied after the forces of each step:
 * NBODY_INTEGRATOR_CPU (default): the reference's CPU order
 *   (ParticleSystem::updateParticlePosition, include/ParticleSystem.h:52-69):
 *   v += a dt/2; x += v dt; a = F; v += a dt/2.
 * NBODY_INTEGRATOR_GPU_EULER: the reference's GLSL path
 *   (src/shaders/ComputeShaders/updateParticles.glsl:44-55): v += F dt; x += v dt.
 *   The accelerations array then holds F (the forces output), which the GLSL
 *   path leaves untouched. Every operation is rounded on its own. */
#define NBODY_INTEGRATOR_CPU 0
#define NBODY_INTEGRATOR_GPU_EULER 1

typedef struct nbody_ctx nbody_ctx;

/* Human-readable name of a status code. */
const char *nbody_status_string(int status);

/* Text of the last CUDA error seen by this context ("" if none). */
const char *nbody_last_error(const nbody_ctx *ctx);

/* Creates a solver for n bodies on CUDA device `device`: time step dt,
 * squared softening eps2 (>= 0), theta2 = squared opening angle for BH
 * (<= 0 selects the reference's 0.25, src/Octree/Octree.cpp:15; ignored for PP).
 * G = 1 as in the reference (ParticleSolverCPUParallel.cpp:9). */
int nbody_create(nbody_ctx **out, int device, int mode, int64_t n, float dt, float eps2, float theta2);
int nbody_destroy(nbody_ctx *ctx);

/* Launch work on `stream` (a cudaStream_t); NULL restores the context's own stream. */
int nbody_set_stream(nbody_ctx *ctx, void *stream);

/* ParticleSolver::getSquaredSoftening (include/ParticleSolver.h:13). */
float nbody_get_squared_softening(const nbody_ctx *ctx);

/* ParticleSolver::updateParticlePositions (include/ParticleSolver.h:12),
 * repeated `steps` times, on host arrays in the ParticleSystem layout: copies
 * positions, velocities, accelerations and masses in, advances, and copies
 * positions, velocities, accelerations (and forces4, which may be NULL) back
 * before returning. forces4 receives the acceleration evaluated at the
 * positions the last step started from, as the reference's forces[] array.
 * Page-locked host memory (cudaHostAlloc / cudaMallocHost, or registered and
 * mapped) is read and written in place by one kernel each way over the
 * host-device link; pageable memory goes through one copy per array. Both
 * move the same values. */
int nbody_update_host(nbody_ctx *ctx, float *positions4, float *velocities4, float *accelerations4,
                      const float *masses4, float *forces4, int steps);

/* 1 when the host-layout calls on `device` would read or write the buffer
 * [p, p + bytes) in place (page-locked, mapped for that device, 16-byte
 * aligned, and page-locked over all `bytes`), 0 when they would copy it
 * through cudaMemcpyAsync instead; NBODY_ERR_ARG for a null pointer or a
 * non-positive size. No counterpart in the reference (its solvers take host
 * arrays only); it lets a caller check that its buffers get the in-place
 * path. */
int nbody_host_in_place(const void *p, int64_t bytes, int device);

/* Resident mode: state stays in HBM between calls. nbody_upload orders its
 * reads of the host arrays on the context's stream: pageable arrays may be
 * reused when it returns, page-locked ones only after the next nbody_sync,
 * nbody_download or nbody_update_host (as with cudaMemcpyAsync). */
int nbody_upload(nbody_ctx *ctx, const float *positions4, const float *velocities4,
                 const float *accelerations4, const float *masses4);
int nbody_step(nbody_ctx *ctx, int steps);
int nbody_download(nbody_ctx *ctx, float *positions4, float *velocities4, float *accelerations4,
                   float *forces4);
/* Masses of the resident state in the reference layout (masses4[4*i] = m_i,
 * other components 0), caller's body order. Masses never change during a run;
 * this is for states made on the device (nbody_init_device). Waits for the
 * context's stream. */
int nbody_download_masses(nbody_ctx *ctx, float *masses4);
/* Waits for the context's stream and returns the device status word
 * (NBODY_OK, or NBODY_ERR_TIMEOUT / NBODY_ERR_CAPACITY raised by a kernel). */
int nbody_sync(nbody_ctx *ctx);

/* Device pointers of the resident state (library layout, see above). A
 * Barnes-Hut context keeps its state in the order of its last Morton sort;
 * nbody_device_order then gives the int array mapping each entry to the
 * caller's body index (NULL while the state is still in the caller's order). */
int nbody_device_state(nbody_ctx *ctx, void **pos_mass4, void **vel4, void **acc4);
int nbody_device_order(nbody_ctx *ctx, void **ids);

/* Direct-sum accelerations for n bodies on device buffers (library layout):
 * force4[i] = sum_j m_j (x_j - x_i) / (|x_j - x_i|^2 + eps2)^1.5, the -v 2
 * force (ParticleSolverCPUParallel.cpp:27-40). Runs on the context's stream,
 * using the context's eps2 and its scratch memory. */
int nbody_pp_forces_device(nbody_ctx *ctx, const void *pos_mass4, void *force4, int64_t n);

/* One direct-sum step on device buffers: forces at pos_in, then the
 * reference integrator (include/ParticleSystem.h:52-69) writing pos_out
 * (pos_in != pos_out), vel4 and acc4 in place; force4 may be NULL. */
int nbody_pp_step_device(nbody_ctx *ctx, const void *pos_in, void *pos_out, void *vel4, void *acc4,
                         void *force4, int64_t n);

/* Launch shape the direct-sum kernel picked for n bodies: i-bodies per
 * thread, j-slices and CTAs. For tests and tuning reports. */
int nbody_pp_config(nbody_ctx *ctx, int64_t n, int *bodies_per_thread, int *slices, int *ctas);

/* Conservation diagnostics of the resident state, computed in FP64 (the only
 * FP64 arithmetic on the GPU; the reference has no diagnostics): out[0]
 * kinetic energy, out[1] potential energy (softened, each pair once; direct sum
 * for a PP context, the Barnes-Hut walk with the context's theta2 for a BH
 * context), out[2..4] linear momentum, out[5..7] angular momentum about the
 * origin. Waits for the context's stream. */
int nbody_diagnostics(nbody_ctx *ctx, double *out);

/* Seeded initial conditions generated on the GPU straight into the resident
 * state, in place of nbody_upload (same effect: the next nbody_step starts from
 * them; body i is caller index i for nbody_download). The reference's
 * initialisers (the files under src/ParticleSystemInitializer/, chosen by -i in
 * src/main.cpp:41-66) seed from the clock or std::random_device; these restate
 * their shapes with a counter-based generator, so a (kind, seed, params, n)
 * always gives the same bits. Kinds 1, 2, 4, 5, 6 keep the reference's -i
 * numbers (include/enums.h:3-11) and take params[0..2] = world dimensions
 * (default 5, 5, 5, the reference's world); a sphere takes params[3] = velocity
 * pattern (0 outward, 1 inward, 2 orbit). The galaxy is the reference's first,
 * fixed-shape branch. Workload kinds (G = 1):
 *   NBODY_INIT_PLUMMER       params = {a, body mass, truncation / a}      default {100, 1, 20}
 *   NBODY_INIT_UNIFORM_BALL  params = {radius, mass lo, mass hi}          default {100, 1, 10}
 *   NBODY_INIT_TWO_DISCS     params = {scale length, scale height, central mass, separation,
 *                                      relative speed, inclination deg, eps2, star mass}
 *                                                       default {200, 20, 1e6, 2000, 50, 30, 40, 1}
 *                            (n even; bodies 0 and n/2 are the central masses)
 * params may be NULL (all defaults); the first nparams (<= NBODY_INIT_MAX_PARAMS)
 * replace the defaults. Enqueued on the context's stream. */
#define NBODY_INIT_CUBE 1
#define NBODY_INIT_GALAXY 2
#define NBODY_INIT_SPHERE 4
#define NBODY_INIT_BALL 5
#define NBODY_INIT_CUBE_SURFACE 6
#define NBODY_INIT_PLUMMER 16
#define NBODY_INIT_UNIFORM_BALL 17
#define NBODY_INIT_TWO_DISCS 18
#define NBODY_INIT_MAX_PARAMS 8
int nbody_init_device(nbody_ctx *ctx, int kind, uint64_t seed, const float *params, int nparams);

/* Selects the integrator (NBODY_INTEGRATOR_*). */
int nbody_set_integrator(nbody_ctx *ctx, int integrator);

/* Selects the key used to build the Barnes-Hut tree (NBODY_KEYS_*). */
int nbody_set_key_mode(nbody_ctx *ctx, int mode);

/* Barnes-Hut pieces on device buffers (context's stream and workspace).
 *
 * nbody_bh_keys_device: the root box of n bodies (min xyz, max xyz; the
 * reference's seeds, src/Octree/ParallelOctreeCPU.cpp:76-118) into box_out
 * (6 floats, device) and their 63-bit keys of the context's key mode
 * (NBODY_KEYS_*) into keys_out (uint64, device).
 *
 * nbody_sort_pairs_device: sorts (uint64 key, uint32 value) pairs by key in
 * place, stably -- replaces src/shaders/ComputeShaders/bitonicSort.glsl:23-50.
 *
 * nbody_bh_forces_device: Barnes-Hut accelerations of n bodies (library
 * layout, caller's order) with the context's eps2 and theta2: the
 * acceleration -v 6 computes (ParticleSolverBHutCPUParallel.cpp:18-46 with
 * Octree::computeGravityForce, src/Octree/Octree.cpp:303-338).
 *
 * nbody_bh_tree_export: the tree of the last Barnes-Hut build, in pre-order:
 * *count records, of which the first min(cap, count) are copied to host as 8
 * floats each (centre of mass x, y, z, mass, then as int32 bit patterns:
 * side^2 (float, -1 for leaves), next record, first body, body count of a
 * leaf); box_host (may be NULL) receives the root box. */
int nbody_bh_keys_device(nbody_ctx *ctx, const void *pos_mass4, int64_t n, void *keys_out, void *box_out);
int nbody_sort_pairs_device(nbody_ctx *ctx, void *keys, void *vals, int64_t n);
int nbody_bh_forces_device(nbody_ctx *ctx, const void *pos_mass4, void *force4, int64_t n);
int nbody_bh_tree_export(nbody_ctx *ctx, float *records_host, int64_t cap, int64_t *count, float *box_host);

/* Barnes-Hut work counters, for measurement: returns (and clears) the number
 * of pairwise force evaluations and of tree records visited by warps since
 * the last call, then enables (enable != 0) or disables counting for later
 * traversals. Counting uses a separate traversal variant; leave it off when
 * timing. */
int nbody_bh_counters(nbody_ctx *ctx, int enable, int64_t *pair_evaluations, int64_t *warp_visits);

/* Per-stage timing. While enabled, every kernel stage launched by this
 * context is bracketed by a CUDA event pair on its launch stream.
 * nbody_profile_read waits for them, writes the summed milliseconds and launch
 * counts of stages 0..nstages-1, and clears the record. Stage names come from
 * nbody_stage_name(0 .. nbody_stage_count()-1). */
int nbody_profile_enable(nbody_ctx *ctx, int on);
int nbody_profile_read(nbody_ctx *ctx, double *ms, int *launches, int nstages);
const char *nbody_stage_name(int stage);
int nbody_stage_count(void);

/* Self-test of the bounded device waits (no counterpart in the reference):
 * runs a kernel on `device` whose mbarrier wait can never complete, through
 * the bounded-wait helper the force kernels use, with a limit of limit_us
 * microseconds (1 .. 1,000,000). The kernel gives up, so the call returns
 * NBODY_OK with *kernel_status = NBODY_ERR_TIMEOUT and *waited_ms (may be
 * NULL) the time it waited; the device stays usable. Synchronises the device. */
int nbody_selftest_wait(int device, int64_t limit_us, int *kernel_status, double *waited_ms);

/* ---------------------------------------------------------------- ensembles
 * Many independent systems of uneven size stepped together on one GPU (no
 * counterpart in the reference, which steps one system per process). Each
 * system keeps the semantics of its solver path: systems with n < crossover
 * (or added with mode NBODY_MODE_PP) use the direct sum of nbody_create(..,
 * NBODY_MODE_PP, ..), the others Barnes-Hut (NBODY_MODE_BH) with their own
 * theta2; every system has its own dt, eps2 and integrator. A system's result
 * does not depend on the other systems in the ensemble: it is the same alone
 * and in any mix, bit for bit. Barnes-Hut systems follow the single-system
 * solver bit for bit; direct-sum systems sum in a different order than the
 * single-system kernel (which splits j-ranges across CTAs).
 *
 * Systems are added and removed between steps; the packed layout is rebuilt at
 * the next call that needs it (upload, init, step, download), moving the
 * states of the remaining systems on the device. Every live system must hold
 * a state (upload or init_device) before a step. nbody_ensemble_step(e, k, g)
 * runs k steps, in CUDA graphs of g steps each when g > 0 (captured once per
 * g and buffer parity, then replayed) and the rest one launch sequence at a
 * time. An ensemble is not re-entrant. */
typedef struct nbody_ensemble nbody_ensemble;
int nbody_ensemble_create(nbody_ensemble **out, int device, int64_t crossover);
int nbody_ensemble_destroy(nbody_ensemble *e);
const char *nbody_ensemble_last_error(const nbody_ensemble *e);
/* Launches go to `stream` (NULL: the ensemble's own); the direct-sum side
 * stream takes that stream's priority. */
int nbody_ensemble_set_stream(nbody_ensemble *e, void *stream);
/* pp_shape: direct-sum launch shape 0 = 128 threads x 2 bodies, 1 = 256 x 2
 * (default), 2 = 256 x 4, 3 = 128 x 4; key_mode: NBODY_KEYS_*. */
int nbody_ensemble_set_options(nbody_ensemble *e, int pp_shape, int key_mode);
/* mode: NBODY_MODE_PP, NBODY_MODE_BH, or -1 (by crossover). */
int nbody_ensemble_add(nbody_ensemble *e, int64_t n, float dt, float eps2, float theta2, int mode, int integrator,
                       int *system);
int nbody_ensemble_remove(nbody_ensemble *e, int system);
int nbody_ensemble_system_info(nbody_ensemble *e, int system, int *mode, int64_t *n);
/* Host arrays in the reference layout, as nbody_upload; returns once they may be reused. */
int nbody_ensemble_upload(nbody_ensemble *e, int system, const float *positions4, const float *velocities4,
                          const float *accelerations4, const float *masses4);
/* As nbody_init_device, for one system (the same bits as a single-system context). */
int nbody_ensemble_init_device(nbody_ensemble *e, int system, int kind, uint64_t seed, const float *params,
                               int nparams);
int nbody_ensemble_step(nbody_ensemble *e, int steps, int graph_steps);
/* Waits for the ensemble's stream; any argument may be NULL. */
int nbody_ensemble_download(nbody_ensemble *e, int system, float *positions4, float *velocities4,
                            float *accelerations4, float *masses4);
int nbody_ensemble_sync(nbody_ensemble *e);
/* Live systems, bodies per group, and kernel launches per step. */
int nbody_ensemble_counts(nbody_ensemble *e, int *systems, int64_t *pp_bodies, int64_t *bh_bodies,
                          int *launches_per_step);
/* Per-stage CUDA-event timing as nbody_profile_enable / nbody_profile_read
 * (stage names from nbody_stage_name); while it is on, steps run without
 * graphs. The direct-sum stage is timed on the side stream. */
int nbody_ensemble_profile_enable(nbody_ensemble *e, int on);
int nbody_ensemble_profile_read(nbody_ensemble *e, double *ms, int *launches, int nstages);
/* Device bytes one system of n bodies takes in an ensemble (for admission). */
int64_t nbody_ensemble_footprint(int64_t n, int mode);

/* Direct-sum accelerations without any allocation by this library. It has
 * no counterpart in the reference. It is for callers that cannot let a library
 * call cudaMalloc: a frame or control loop that must not stall on an
 * allocation (cudaMalloc / cudaFree can synchronise the device), or a host
 * application that owns all device memory through its own pool. Same result
 * as nbody_pp_forces_device (library layout, G = 1, squared softening eps2),
 * enqueued on `stream` (a cudaStream_t; NULL = the legacy default stream) of
 * the current device.
 *
 * Scratch: a fixed 8 MiB array in device memory inside this library, held on
 * every GPU that loads it until the process exits; nothing else is
 * allocated, by the library or on its behalf. n > NBODY_NOALLOC_MAX_BODIES
 * returns NBODY_ERR_CAPACITY; for large n fewer j-slices are used so that
 * the partial sums fit. The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress); make that first call before any stream
 * capture. Every call shares the one array: calls whose work overlaps on the
 * GPU (several streams or host threads) race and must be serialised by the
 * caller.
 *
 * kernel_status may be NULL; if given, the call waits for `stream` and
 * stores the kernel's status there (NBODY_OK, or NBODY_ERR_TIMEOUT). */
#define NBODY_NOALLOC_MAX_BODIES 4194304
int nbody_pp_forces_noalloc(const void *pos_mass4, void *force4, int64_t n, float eps2, void *stream,
                            int *kernel_status);

#ifdef __cplusplus
}
#endif

#endif /* NBODY_GB300_H */
