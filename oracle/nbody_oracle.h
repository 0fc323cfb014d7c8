/* CPU oracle for the per-step gravity solve: a plain-C restatement of the
 * reference's CPU solvers (direct sum -v 2, Barnes-Hut -v 6) plus the
 * 63-bit Morton key / stable sort restatement and an FP64 direct-sum checker.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load this library, and only as
 * the checker or the timed CPU baseline; the product never links or calls it.
 *
 * Layout conventions (reference include/ParticleSystem.h:100-104): pos4, vel4,
 * acc4, force4 are float[4*n] (x, y, z, w) arrays; w of positions is 0 in the
 * reference; masses are a separate float[n] array (the reference stores them in
 * masses[i].x).
 */
#ifndef NBODY_ORACLE_H
#define NBODY_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    ORC_OK = 0,
    ORC_ERR_ARG = 1,
    ORC_ERR_CAPACITY = 4, /* a -v 6 task bucket or subtree region overflowed */
    ORC_ERR_NOMEM = 5
};

int orc_version(void);

/* Root box of -v 6 (src/Octree/ParallelOctreeCPU.cpp:76-118). */
void orc_bbox(int64_t n, const float *pos4, float bmin[3], float bmax[3]);

/* 63-bit Morton keys, 21 bits per axis, x highest in each bit triple. */
uint64_t orc_morton63_key(float px, float py, float pz, const float bmin[3], const float bmax[3]);
void orc_morton63(int64_t n, const float *pos4, const float bmin[3], const float bmax[3], uint64_t *keys);

/* Keys from the reference's octree descent (Octree::getNextNode), 21 levels. */
uint64_t orc_octree_key(float px, float py, float pz, const float bmin[3], const float bmax[3]);
void orc_octree_keys(int64_t n, const float *pos4, const float bmin[3], const float bmax[3], uint64_t *keys);

/* Stable LSD radix argsort of 64-bit keys: perm[r] = index of the r-th smallest
 * key, ties kept in index order. keys_sorted may be NULL. */
int orc_sort_stable(int64_t n, const uint64_t *keys, uint64_t *keys_sorted, uint32_t *perm);

/* -v 2 force (src/ParticleSolver/ParticleSolverCPUParallel/ParticleSolverCPUParallel.cpp:27-40). */
void orc_pp_forces(int64_t n, const float *pos4, const float *mass, float eps2, float *force4, int threads);

/* Reference integrator (include/ParticleSystem.h:52-69). */
void orc_integrate(int64_t n, float *pos4, float *vel4, float *acc4, const float *force4, float dt, int threads);

/* `steps` x (-v 2 force, integrate). Returns seconds spent. */
double orc_pp_run(int64_t n, float *pos4, float *vel4, float *acc4, const float *mass, float *force4,
                  float dt, float eps2, int steps, int threads);

/* `steps` x -v 6 step (reset, insert, traversal, integrate).
 * theta2 <= 0 selects the reference default 0.25. patched = 0 keeps the
 * reference's per-task capacities (n/2 nodes per subtree, 0.6 * n/2 bodies per
 * task) and reports ORC_ERR_CAPACITY where the reference would overflow;
 * patched = 1 sizes every subtree region from its body count.
 * Outputs (may be NULL): seconds, root mass after the last build, node count. */
int orc_bh_run(int64_t n, float *pos4, float *vel4, float *acc4, const float *mass, float *force4,
               float dt, float eps2, float theta2, int steps, int threads, int patched,
               double *seconds, float *root_mass, int64_t *nodes_used);

/* One -v 6 tree build (reference capacities); copies up to cap nodes as 12
 * floats (mass, first_child, next, com.xyz, min.xyz, max.xyz). Returns the pool
 * size, or a negated ORC_ERR_* code. */
int64_t orc_bh_tree(int64_t n, const float *pos4, const float *mass, float *out, int64_t cap);

/* FP64 direct sum for the k bodies listed in idx (all bodies when idx is NULL
 * and k == n), self term excluded: acc64[3*t..] for target t. */
void orc_direct_f64(int64_t n, const float *pos4, const float *mass, double eps2,
                    const int64_t *idx, int64_t k, double *acc64, int threads);

/* FP64 conservation diagnostics: out[0] kinetic, out[1] potential (softened,
 * pairs counted once), out[2..4] linear momentum, out[5..7] angular momentum. */
void orc_diagnostics_f64(int64_t n, const float *pos4, const float *vel4, const float *mass,
                         double eps2, double out[8], int threads);

#ifdef __cplusplus
}
#endif
#endif
