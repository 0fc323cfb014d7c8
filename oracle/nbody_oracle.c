/* CPU oracle: plain-C restatement of the reference's CPU gravity solve.
 *
 * TEST INFRASTRUCTURE ONLY (see nbody_oracle.h). Each function cites the
 * reference file:line it restates. Arithmetic is written in the same order as
 * the reference (component-wise vec4 operations, pow(x, 1.5f), a divide) and
 * the library is compiled with the reference's release flags (-O3 -ffast-math
 * -fopenmp), so that its results track the reference's own binary; where it
 * deviates on purpose it says so:
 *   - node indices are 64-bit integers, not floats (include/Node.h:16-30 stores
 *     them as float, which rounds once indices pass 2^24);
 *   - bodies are bucketed into -v 6 tasks in ascending body order (the
 *     reference appends under per-leaf locks, so its order within a task varies
 *     from run to run; a one-thread reference run has exactly this order);
 *   - a bucket or subtree region that would overflow is reported as
 *     ORC_ERR_CAPACITY instead of writing past its end.
 */
#define _DEFAULT_SOURCE
#include "nbody_oracle.h"

#include <float.h>
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>

int orc_version(void) { return 1; }

static void set_threads(int threads) {
    if (threads > 0) omp_set_num_threads(threads);
}

/* ---- component-wise vec4, as used by the reference through glm ---------- */
typedef struct { float x, y, z, w; } v4;
static inline v4 v4_make(float x, float y, float z, float w) { v4 r = {x, y, z, w}; return r; }
static inline v4 v4_load(const float *p) { return v4_make(p[0], p[1], p[2], p[3]); }
static inline v4 v4_add(v4 a, v4 b) { return v4_make(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
static inline v4 v4_sub(v4 a, v4 b) { return v4_make(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
static inline v4 v4_scale(v4 a, float s) { return v4_make(a.x * s, a.y * s, a.z * s, a.w * s); }
static inline v4 v4_div(v4 a, float s) { return v4_make(a.x / s, a.y / s, a.z / s, a.w / s); }
static inline float v4_len2(v4 a) { return a.x * a.x + a.y * a.y + a.z * a.z + a.w * a.w; }
static inline void v4_store(float *p, v4 a) { p[0] = a.x; p[1] = a.y; p[2] = a.z; p[3] = a.w; }

/* ---- bounding box: src/Octree/ParallelOctreeCPU.cpp:76-118 --------------
 * min seeds are FLT_MAX; max seeds are FLT_MIN (the smallest positive normal,
 * numeric_limits<float>::min(), :80), so an axis whose coordinates are all
 * negative keeps max = FLT_MIN. Strict comparisons as at :89-106. */
void orc_bbox(int64_t n, const float *pos4, float bmin[3], float bmax[3]) {
    float mnx = FLT_MAX, mny = FLT_MAX, mnz = FLT_MAX;
    float mxx = FLT_MIN, mxy = FLT_MIN, mxz = FLT_MIN;
    for (int64_t i = 0; i < n; ++i) {
        const float x = pos4[4 * i], y = pos4[4 * i + 1], z = pos4[4 * i + 2];
        if (x < mnx) mnx = x;
        if (y < mny) mny = y;
        if (z < mnz) mnz = z;
        if (x > mxx) mxx = x;
        if (y > mxy) mxy = y;
        if (z > mxz) mxz = z;
    }
    bmin[0] = mnx; bmin[1] = mny; bmin[2] = mnz;
    bmax[0] = mxx; bmax[1] = mxy; bmax[2] = mxz;
}

/* ---- -v 2 direct sum -----------------------------------------------------
 * src/ParticleSolver/ParticleSolverCPUParallel/ParticleSolverCPUParallel.cpp:27-40,
 * OpenMP static over i (:14-16), G = 1 (:9). */
void orc_pp_forces(int64_t n, const float *pos4, const float *mass, float eps2, float *force4, int threads) {
    set_threads(threads);
    const float G = 1.0f;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const v4 pi = v4_load(pos4 + 4 * i);
        v4 total = v4_make(0.f, 0.f, 0.f, 0.f);
        for (int64_t j = 0; j < n; ++j) {
            if (i != j) {
                const v4 r = v4_sub(v4_load(pos4 + 4 * j), pi);
                const float dist = powf(v4_len2(r) + eps2, 1.5f);
                total = v4_add(total, v4_scale(r, (G * mass[j]) / dist));
            }
        }
        v4_store(force4 + 4 * i, total);
    }
}

/* ---- integrator: include/ParticleSystem.h:52-69 ---------------------------
 * v += a*dt/2; x += v*dt; a = F; v += a*dt/2 (all four components). */
void orc_integrate(int64_t n, float *pos4, float *vel4, float *acc4, const float *force4, float dt, int threads) {
    set_threads(threads);
    const float h = dt * 0.5f;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        v4 v = v4_load(vel4 + 4 * i);
        v4 x = v4_load(pos4 + 4 * i);
        v4 a = v4_load(acc4 + 4 * i);
        v = v4_add(v, v4_scale(a, h));
        x = v4_add(x, v4_scale(v, dt));
        a = v4_load(force4 + 4 * i);
        v = v4_add(v, v4_scale(a, h));
        v4_store(vel4 + 4 * i, v);
        v4_store(pos4 + 4 * i, x);
        v4_store(acc4 + 4 * i, a);
    }
}

double orc_pp_run(int64_t n, float *pos4, float *vel4, float *acc4, const float *mass, float *force4,
                  float dt, float eps2, int steps, int threads) {
    double secs = 0.0;
    for (int s = 0; s < steps; ++s) {
        const double t0 = omp_get_wtime();
        orc_pp_forces(n, pos4, mass, eps2, force4, threads);
        orc_integrate(n, pos4, vel4, acc4, force4, dt, threads);
        secs += omp_get_wtime() - t0;
    }
    return secs;
}

/* ---- -v 6 Barnes-Hut -------------------------------------------------------
 * Node: include/Node.h:7-93 with integer links. Leaf <=> first_child < 0;
 * occupied <=> mass > 0; an empty leaf has mass -1. */
typedef struct {
    float mass;
    float com[3];
    float mn[3];
    float mx[3];
    int64_t first_child;
    int64_t next;
} onode;

typedef struct {
    onode *nodes;
    size_t map_bytes;
    int64_t father_nodes;   /* maxNodes  (ParallelOctreeCPU.cpp:7-23)          */
    int father_depth;       /* maxDepth                                        */
    int64_t tasks;          /* totalTasks = 8^maxDepth (:35)                   */
    int64_t *region;        /* first node of each task's subtree region        */
    int64_t *region_cap;    /* nodes available in each region                  */
    int64_t *node_count;    /* nodeCounts[t]                                   */
    int64_t **sub_parents;  /* subTreeParents, per task, creation order        */
    int64_t *parent_count;  /* parentCounts[t]                                 */
    int64_t *parent_cap;
    int64_t *parents;       /* father-level parent list                        */
    int64_t parent_n;
    int64_t node_total;     /* father nodes + father subdivisions count        */
    int error;
} otree;

/* Octree::subdivide / ParallelOctreeCPU::subdivide child boxes
 * (src/Octree/Octree.cpp:159-231, ParallelOctreeCPU.cpp:427-497): bit set on
 * an axis selects the lower half [min, min + w/2], bit clear the upper half
 * [min + w/2, max]. Children are linked by next; the last child's next is the
 * parent's next. */
static void make_children(onode *nodes, int64_t parent, int64_t first) {
    onode *p = &nodes[parent];
    p->first_child = first;
    const float w = p->mx[0] - p->mn[0];
    const float h = p->mx[1] - p->mn[1];
    const float d = p->mx[2] - p->mn[2];
    for (int j = 0; j < 8; ++j) {
        onode *c = &nodes[first + j];
        if (j & 4) { c->mn[2] = p->mn[2]; c->mx[2] = p->mn[2] + (d / 2.f); }
        else       { c->mn[2] = p->mn[2] + (d / 2.f); c->mx[2] = p->mx[2]; }
        if (j & 2) { c->mn[1] = p->mn[1]; c->mx[1] = p->mn[1] + (h / 2.f); }
        else       { c->mn[1] = p->mn[1] + (h / 2.f); c->mx[1] = p->mx[1]; }
        if (j & 1) { c->mn[0] = p->mn[0]; c->mx[0] = p->mn[0] + (w / 2.f); }
        else       { c->mn[0] = p->mn[0] + (w / 2.f); c->mx[0] = p->mx[0]; }
        c->mass = -1.f;
        c->first_child = -1;
        if (j < 7) c->next = first + j + 1;
    }
    nodes[first + 7].next = p->next;
}

/* Octree::getNextNode (src/Octree/Octree.cpp:148-153) with
 * Node::getQuadrantCenter (include/Node.h:85-92). */
static inline int64_t next_node(const onode *nodes, const float pos[3], int64_t i) {
    const onode *n = &nodes[i];
    const float cx = n->mn[0] + ((n->mx[0] - n->mn[0]) / 2.f);
    const float cy = n->mn[1] + ((n->mx[1] - n->mn[1]) / 2.f);
    const float cz = n->mn[2] + ((n->mx[2] - n->mn[2]) / 2.f);
    const int q = (pos[0] < cx) | (pos[1] < cy) << 1 | (pos[2] < cz) << 2;
    return n->first_child + q;
}

static void tree_free(otree *t) {
    if (t->nodes) munmap(t->nodes, t->map_bytes);
    if (t->sub_parents) {
        for (int64_t k = 0; k < t->tasks; ++k) free(t->sub_parents[k]);
    }
    free(t->sub_parents);
    free(t->region); free(t->region_cap); free(t->node_count);
    free(t->parent_count); free(t->parent_cap); free(t->parents);
    memset(t, 0, sizeof(*t));
}

/* Father-tree sizing: ParallelOctreeCPU::ParallelOctreeCPU (:7-57). */
static void father_sizing(int64_t n, int64_t *father_nodes, int *depth, int64_t *tasks) {
    int64_t m = 0;
    int d = -1;
    int64_t p8 = 1;
    while (m < n && d < 3) {
        const int64_t tmp = m + p8;
        if (tmp >= n) break;
        m = tmp;
        d++;
        p8 *= 8;
    }
    *father_nodes = m;
    *depth = d;
    *tasks = d < 0 ? 0 : (int64_t)1 << (3 * d);
}

/* ParallelOctreeCPU::insert(pos, mass, subTreeId) (:362-424) including the
 * merge rule (:396-402): two bodies that still share a child after the split
 * merge into one leaf when their squared distance is below 1e-3 or after ten
 * further splits; the merged leaf sits at the newly inserted body's position
 * with the summed mass. */
static int subtree_insert(otree *t, int64_t task, const float pos[3], float m) {
    onode *nodes = t->nodes;
    const int64_t root = t->region[task];
    int64_t i = root;
    for (;;) {
        onode *node = &nodes[i];
        const int leaf = node->first_child < 0;
        if (leaf && !(node->mass > 0.f)) {
            node->com[0] = pos[0]; node->com[1] = pos[1]; node->com[2] = pos[2];
            node->mass = m;
            return ORC_OK;
        }
        if (leaf) {
            const float pos2[3] = {node->com[0], node->com[1], node->com[2]};
            const float m2 = node->mass;
            int64_t split = i;
            for (int guard = 0;; ++guard) {
                if (t->node_count[task] + 8 > t->region_cap[task]) return ORC_ERR_CAPACITY;
                if (t->parent_count[task] >= t->parent_cap[task]) return ORC_ERR_CAPACITY;
                t->sub_parents[task][t->parent_count[task]++] = split;
                const int64_t first = t->node_count[task] + root;
                t->node_count[task] += 8;
                make_children(nodes, split, first);
                const int64_t c1 = next_node(nodes, pos, split);
                const int64_t c2 = next_node(nodes, pos2, split);
                if (c1 != c2) {
                    nodes[c1].com[0] = pos[0]; nodes[c1].com[1] = pos[1]; nodes[c1].com[2] = pos[2];
                    nodes[c1].mass = m;
                    nodes[c2].com[0] = pos2[0]; nodes[c2].com[1] = pos2[1]; nodes[c2].com[2] = pos2[2];
                    nodes[c2].mass = m2;
                    return ORC_OK;
                }
                const v4 dv = v4_sub(v4_make(pos2[0], pos2[1], pos2[2], 0.f), v4_make(pos[0], pos[1], pos[2], 0.f));
                const float dist = v4_len2(dv);
                if (dist < 1e-3f || guard == 10) {
                    nodes[c1].com[0] = pos[0]; nodes[c1].com[1] = pos[1]; nodes[c1].com[2] = pos[2];
                    nodes[c1].mass = m2 + m;
                    return ORC_OK;
                }
                split = c1;
            }
        }
        i = next_node(nodes, pos, i);
    }
}

/* Bottom-up mass / centre of mass over a parent list in reverse creation order
 * (ParallelOctreeCPU::propagate(int), :325-349; Octree::propagate,
 * src/Octree/Octree.cpp:238-258). Occupied children only. */
static void propagate_list(onode *nodes, const int64_t *list, int64_t count) {
    for (int64_t k = count - 1; k >= 0; --k) {
        onode *p = &nodes[list[k]];
        v4 com = v4_make(0.f, 0.f, 0.f, 0.f);
        float mass = 0.f;
        for (int j = 0; j < 8; ++j) {
            const onode *c = &nodes[p->first_child + j];
            if (!(c->mass > 0.f)) continue;
            com = v4_add(com, v4_scale(v4_make(c->com[0], c->com[1], c->com[2], 0.f), c->mass));
            mass += c->mass;
        }
        const v4 r = v4_div(com, mass);
        p->com[0] = r.x; p->com[1] = r.y; p->com[2] = r.z;
        p->mass = mass;
    }
}

/* Relink first_child / next to occupied children only, parents in creation
 * order (ParallelOctreeCPU::prune(int), :293-323; Octree::prune,
 * src/Octree/Octree.cpp:264-294). */
static void prune_list(onode *nodes, const int64_t *list, int64_t count) {
    for (int64_t k = 0; k < count; ++k) {
        onode *p = &nodes[list[k]];
        if (!(p->mass > 0.f)) { p->first_child = p->next; continue; }
        int64_t first = -1, last = -1;
        for (int j = 0; j < 8; ++j) {
            const int64_t c = p->first_child + j;
            if (nodes[c].mass > 0.f) {
                if (first == -1) { first = c; last = c; continue; }
                nodes[last].next = c;
                last = c;
            }
        }
        nodes[last].next = p->next;
        p->first_child = first;
    }
}

/* Octree::computeGravityForce (src/Octree/Octree.cpp:303-338): stackless walk;
 * accept a node if it is a leaf or s^2 < theta * d^2 (s = max side of the
 * node's box, theta the squared opening angle); an accepted occupied node with
 * d^2 > 0 contributes m * r / (d^2 + eps^2)^1.5. */
static void bh_force(const onode *nodes, v4 pos, float eps2, float theta2, float *out) {
    const float G = 1.0f;
    v4 force = v4_make(0.f, 0.f, 0.f, 0.f);
    int64_t i = 0;
    while (i >= 0) {
        const onode *node = &nodes[i];
        const v4 size = v4_sub(v4_make(node->mx[0], node->mx[1], node->mx[2], 0.f),
                               v4_make(node->mn[0], node->mn[1], node->mn[2], 0.f));
        const float sxy = size.x < size.y ? size.y : size.x;
        const float s = sxy < size.z ? size.z : sxy;
        const float s2 = s * s;
        const v4 r = v4_sub(v4_make(node->com[0], node->com[1], node->com[2], 0.f), pos);
        const float d2 = v4_len2(r);
        if (node->first_child < 0 || s2 < theta2 * d2) {
            if (node->mass > 0.f && d2 > 0.f) {
                const float eff = d2 + eps2;
                const float inv = 1.0f / powf(eff, 1.5f);
                force = v4_add(force, v4_scale(v4_scale(r, G * node->mass), inv));
            }
            i = node->next;
        } else {
            i = node->first_child;
        }
    }
    v4_store(out, force);
}

static int tree_alloc(otree *t, int64_t n, int patched, const int64_t *bucket_count) {
    father_sizing(n, &t->father_nodes, &t->father_depth, &t->tasks);
    if (t->tasks <= 0) return ORC_ERR_CAPACITY; /* reference sizes no node for n <= 1 */
    const int64_t per_subtree = n / 2;          /* maxNodesPerSubtree = n/2.0 (:27) */
    t->region = calloc((size_t)t->tasks, sizeof(int64_t));
    t->region_cap = calloc((size_t)t->tasks, sizeof(int64_t));
    t->node_count = calloc((size_t)t->tasks, sizeof(int64_t));
    t->parent_count = calloc((size_t)t->tasks, sizeof(int64_t));
    t->parent_cap = calloc((size_t)t->tasks, sizeof(int64_t));
    t->sub_parents = calloc((size_t)t->tasks, sizeof(int64_t *));
    t->parents = calloc((size_t)(t->father_nodes + t->tasks + 1), sizeof(int64_t));
    if (!t->region || !t->region_cap || !t->node_count || !t->parent_count || !t->parent_cap ||
        !t->sub_parents || !t->parents)
        return ORC_ERR_NOMEM;
    int64_t total = t->father_nodes;
    for (int64_t k = 0; k < t->tasks; ++k) {
        /* reference: region k starts at maxNodes + maxNodesPerSubtree * k (:499-505) */
        const int64_t cap = patched ? 1 + 88 * bucket_count[k] : per_subtree;
        t->region[k] = total;
        t->region_cap[k] = cap;
        t->parent_cap[k] = patched ? 11 * bucket_count[k] + 1 : per_subtree;
        total += cap;
    }
    t->node_total = total;
    t->map_bytes = sizeof(onode) * (size_t)(total > 0 ? total : 1);
    void *p = mmap(NULL, t->map_bytes, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
    if (p == MAP_FAILED) { t->nodes = NULL; return ORC_ERR_NOMEM; }
    t->nodes = (onode *)p;
    for (int64_t k = 0; k < t->tasks; ++k) {
        const int64_t pc = t->parent_cap[k] > 0 ? t->parent_cap[k] : 1;
        t->sub_parents[k] = malloc(sizeof(int64_t) * (size_t)pc);
        if (!t->sub_parents[k]) return ORC_ERR_NOMEM;
    }
    return ORC_OK;
}

/* One -v 6 tree build: ParallelOctreeCPU::reset (:76-118) + insert (:124-206). */
static int tree_build(otree *t, int64_t n, const float *pos4, const float *mass,
                      const int64_t *bucket_start, const int64_t *bucket_body) {
    onode *nodes = t->nodes;
    float bmin[3], bmax[3];
    orc_bbox(n, pos4, bmin, bmax);
    onode *root = &nodes[0];
    root->mn[0] = bmin[0]; root->mn[1] = bmin[1]; root->mn[2] = bmin[2];
    root->mx[0] = bmax[0]; root->mx[1] = bmax[1]; root->mx[2] = bmax[2];
    root->first_child = -1;
    root->mass = -1.f;
    root->next = -1;
    /* Father tree: Octree::subdivide on nodes 0, 1, 2, ... until maxNodes
     * exist (:129-132); parents are recorded in that order. */
    int64_t count = 1;
    t->parent_n = 0;
    for (int64_t p = 0; count < t->father_nodes; ++p) {
        t->parents[t->parent_n++] = p;
        make_children(nodes, p, count);
        count += 8;
    }
    int err = ORC_OK;
    /* Per-task serial insertion + propagate (:158-189), dynamic schedule. */
#pragma omp parallel for schedule(dynamic)
    for (int64_t k = 0; k < t->tasks; ++k) {
        const int64_t leaf = t->father_nodes - t->tasks + k;   /* father leaf owning task k */
        const int64_t task = leaf % t->tasks;
        const int64_t sroot = t->region[task];
        const int64_t b0 = bucket_start[task], b1 = bucket_start[task + 1];
        /* A task that no body reached is skipped (the reference skips tasks
         * whose root was never recorded, :160); its region is unreachable. */
        if (b1 <= b0) continue;
        onode *oct = &nodes[sroot];
        oct->mn[0] = nodes[leaf].mn[0]; oct->mn[1] = nodes[leaf].mn[1]; oct->mn[2] = nodes[leaf].mn[2];
        oct->mx[0] = nodes[leaf].mx[0]; oct->mx[1] = nodes[leaf].mx[1]; oct->mx[2] = nodes[leaf].mx[2];
        oct->first_child = -1;
        oct->mass = -1.f;
        t->node_count[task] = 1;
        t->parent_count[task] = 0;
        oct->next = nodes[leaf].next;
        nodes[leaf].first_child = sroot;
        for (int64_t b = b0; b < b1; ++b) {
            const int64_t j = bucket_body[b];
            const float p[3] = {pos4[4 * j], pos4[4 * j + 1], pos4[4 * j + 2]};
            const int rc = subtree_insert(t, task, p, mass[j]);
            if (rc != ORC_OK) {
#pragma omp atomic write
                err = rc;
                break;
            }
        }
        propagate_list(nodes, t->sub_parents[task], t->parent_count[task]);
    }
    if (err != ORC_OK) return err;
    /* Father leaves that received bodies become parents (:187-192). */
    const int64_t nfather_parents = t->parent_n;
    for (int64_t i = t->father_nodes - t->tasks; i < t->father_nodes; ++i)
        if (bucket_start[i % t->tasks + 1] > bucket_start[i % t->tasks]) t->parents[t->parent_n++] = i;
    /* ParallelOctreeCPU::propagate (:264-291): father leaves copy their
     * subtree root, then father internals combine their eight children. */
    for (int64_t k = t->parent_n - 1; k >= nfather_parents; --k) {
        onode *p = &nodes[t->parents[k]];
        const onode *c = &nodes[p->first_child];
        if (!(c->mass > 0.f)) continue;
        p->com[0] = c->com[0]; p->com[1] = c->com[1]; p->com[2] = c->com[2];
        p->mass = c->mass;
    }
    propagate_list(nodes, t->parents, nfather_parents);
    /* ParallelOctreeCPU::prune (:209-258). */
    prune_list(nodes, t->parents, nfather_parents);
    for (int64_t i = t->father_nodes - t->tasks; i < t->father_nodes; ++i)
        if (nodes[i].mass > 0.f) nodes[nodes[i].first_child].next = nodes[i].next;
#pragma omp parallel for schedule(dynamic)
    for (int64_t k = 0; k < t->tasks; ++k) {
        if (bucket_start[k + 1] <= bucket_start[k]) continue;
        prune_list(nodes, t->sub_parents[k], t->parent_count[k]);
    }
    return ORC_OK;
}

/* Bucket bodies into father leaves (:134-152) in ascending body order. */
static void bucket_bodies(int64_t n, const float *pos4, const onode *nodes, int depth, int64_t tasks,
                          int64_t *task_of, int64_t *bucket_start, int64_t *bucket_body) {
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < n; ++j) {
        const float p[3] = {pos4[4 * j], pos4[4 * j + 1], pos4[4 * j + 2]};
        int64_t i = 0;
        for (int d = 0; d < depth; ++d) i = next_node(nodes, p, i);
        task_of[j] = i % tasks;
    }
    memset(bucket_start, 0, sizeof(int64_t) * (size_t)(tasks + 1));
    for (int64_t j = 0; j < n; ++j) bucket_start[task_of[j] + 1]++;
    for (int64_t k = 0; k < tasks; ++k) bucket_start[k + 1] += bucket_start[k];
    int64_t *fill = malloc(sizeof(int64_t) * (size_t)tasks);
    memcpy(fill, bucket_start, sizeof(int64_t) * (size_t)tasks);
    for (int64_t j = 0; j < n; ++j) bucket_body[fill[task_of[j]]++] = j;
    free(fill);
}

/* Father tree only, used to bucket bodies before the tree exists (the
 * reference descends the freshly subdivided father tree, :136-145). */
static void father_only(onode *nodes, int64_t father_nodes, const float bmin[3], const float bmax[3]) {
    onode *root = &nodes[0];
    root->mn[0] = bmin[0]; root->mn[1] = bmin[1]; root->mn[2] = bmin[2];
    root->mx[0] = bmax[0]; root->mx[1] = bmax[1]; root->mx[2] = bmax[2];
    root->first_child = -1;
    root->mass = -1.f;
    root->next = -1;
    int64_t count = 1;
    for (int64_t p = 0; count < father_nodes; ++p) {
        make_children(nodes, p, count);
        count += 8;
    }
}

static int counts_fit(const otree *t, const int64_t *bucket_start) {
    for (int64_t k = 0; k < t->tasks; ++k)
        if (1 + 88 * (bucket_start[k + 1] - bucket_start[k]) > t->region_cap[k]) return 0;
    return 1;
}

int orc_bh_run(int64_t n, float *pos4, float *vel4, float *acc4, const float *mass, float *force4,
               float dt, float eps2, float theta2, int steps, int threads, int patched,
               double *seconds, float *root_mass, int64_t *nodes_used) {
    set_threads(threads);
    if (theta2 <= 0.f) theta2 = 0.5f * 0.5f;   /* src/Octree/Octree.cpp:15 */
    if (seconds) *seconds = 0.0;
    int64_t fnodes, tasks;
    int depth;
    father_sizing(n, &fnodes, &depth, &tasks);
    if (tasks <= 0 || n < 2) return ORC_ERR_ARG;  /* the reference allocates no node here */
    int64_t *task_of = malloc(sizeof(int64_t) * (size_t)n);
    int64_t *bucket_start = malloc(sizeof(int64_t) * (size_t)(tasks + 1));
    int64_t *bucket_body = malloc(sizeof(int64_t) * (size_t)n);
    int64_t *counts = malloc(sizeof(int64_t) * (size_t)tasks);
    onode *fat = calloc((size_t)fnodes, sizeof(onode));
    if (!task_of || !bucket_start || !bucket_body || !counts || !fat) {
        free(task_of); free(bucket_start); free(bucket_body); free(counts); free(fat);
        return ORC_ERR_NOMEM;
    }
    int rc = ORC_OK;
    const int64_t per_task_bodies = (int64_t)((double)(n / 2) * 0.6);  /* maxParticlesPerTask (:50) */
    otree t;
    memset(&t, 0, sizeof(t));
    int have_tree = 0;
    for (int s = 0; s < steps && rc == ORC_OK; ++s) {
        const double t0 = omp_get_wtime();
        double t_alloc = 0.0;
        float bmin[3], bmax[3];
        orc_bbox(n, pos4, bmin, bmax);
        father_only(fat, fnodes, bmin, bmax);
        bucket_bodies(n, pos4, fat, depth, tasks, task_of, bucket_start, bucket_body);
        if (!patched) {
            for (int64_t k = 0; k < tasks; ++k)
                if (bucket_start[k + 1] - bucket_start[k] > per_task_bodies) rc = ORC_ERR_CAPACITY;
            if (rc != ORC_OK) break;
        }
        /* The node pool is sized once, as in the reference's constructor
         * (ParallelOctreeCPU.cpp:38); its set-up time is not counted. A patched
         * pool is re-sized only when a region's body count outgrows it. */
        if (!have_tree || (patched && !counts_fit(&t, bucket_start))) {
            const double a0 = omp_get_wtime();
            if (have_tree) tree_free(&t);
            for (int64_t k = 0; k < tasks; ++k) counts[k] = 2 * (bucket_start[k + 1] - bucket_start[k]) + 4;
            rc = tree_alloc(&t, n, patched, counts);
            have_tree = rc == ORC_OK;
            t_alloc = omp_get_wtime() - a0;
            if (rc != ORC_OK) break;
        }
        rc = tree_build(&t, n, pos4, mass, bucket_start, bucket_body);
        if (rc == ORC_OK) {
            if (root_mass) *root_mass = t.nodes[0].mass;
            if (nodes_used) {
                int64_t used = t.father_nodes;
                for (int64_t k = 0; k < t.tasks; ++k)
                    if (bucket_start[k + 1] > bucket_start[k]) used += t.node_count[k];
                *nodes_used = used;
            }
            const onode *nodes = t.nodes;
#pragma omp parallel for schedule(dynamic)
            for (int64_t i = 0; i < n; ++i)
                bh_force(nodes, v4_load(pos4 + 4 * i), eps2, theta2, force4 + 4 * i);
            orc_integrate(n, pos4, vel4, acc4, force4, dt, threads);
        }
        if (seconds) *seconds += omp_get_wtime() - t0 - t_alloc;
    }
    if (have_tree) tree_free(&t);
    free(task_of); free(bucket_start); free(bucket_body); free(counts); free(fat);
    return rc;
}

int64_t orc_bh_tree(int64_t n, const float *pos4, const float *mass, float *out, int64_t cap) {
    int64_t fnodes, tasks;
    int depth;
    father_sizing(n, &fnodes, &depth, &tasks);
    if (tasks <= 0 || n < 2) return -ORC_ERR_ARG;
    int64_t *task_of = malloc(sizeof(int64_t) * (size_t)n);
    int64_t *bucket_start = malloc(sizeof(int64_t) * (size_t)(tasks + 1));
    int64_t *bucket_body = malloc(sizeof(int64_t) * (size_t)n);
    onode *fat = calloc((size_t)fnodes, sizeof(onode));
    float bmin[3], bmax[3];
    orc_bbox(n, pos4, bmin, bmax);
    father_only(fat, fnodes, bmin, bmax);
    bucket_bodies(n, pos4, fat, depth, tasks, task_of, bucket_start, bucket_body);
    otree t;
    memset(&t, 0, sizeof(t));
    int rc = tree_alloc(&t, n, 0, NULL);
    if (rc == ORC_OK) rc = tree_build(&t, n, pos4, mass, bucket_start, bucket_body);
    int64_t total = rc == ORC_OK ? t.node_total : -rc;
    if (rc == ORC_OK) {
        for (int64_t i = 0; i < total && i < cap; ++i) {
            const onode *d = &t.nodes[i];
            float *o = out + 12 * i;
            o[0] = d->mass; o[1] = (float)d->first_child; o[2] = (float)d->next;
            o[3] = d->com[0]; o[4] = d->com[1]; o[5] = d->com[2];
            o[6] = d->mn[0]; o[7] = d->mn[1]; o[8] = d->mn[2];
            o[9] = d->mx[0]; o[10] = d->mx[1]; o[11] = d->mx[2];
        }
    }
    tree_free(&t);
    free(task_of); free(bucket_start); free(bucket_body); free(fat);
    return total;
}

/* ---- FP64 checkers ---------------------------------------------------------- */
void orc_direct_f64(int64_t n, const float *pos4, const float *mass, double eps2,
                    const int64_t *idx, int64_t k, double *acc64, int threads) {
    set_threads(threads);
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t t = 0; t < k; ++t) {
        const int64_t i = idx ? idx[t] : t;
        const double xi = pos4[4 * i], yi = pos4[4 * i + 1], zi = pos4[4 * i + 2];
        double ax = 0.0, ay = 0.0, az = 0.0;
        for (int64_t j = 0; j < n; ++j) {
            if (j == i) continue;
            const double dx = (double)pos4[4 * j] - xi;
            const double dy = (double)pos4[4 * j + 1] - yi;
            const double dz = (double)pos4[4 * j + 2] - zi;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            const double w = (double)mass[j] / (r2 * sqrt(r2));
            ax += w * dx; ay += w * dy; az += w * dz;
        }
        acc64[3 * t] = ax; acc64[3 * t + 1] = ay; acc64[3 * t + 2] = az;
    }
}

void orc_diagnostics_f64(int64_t n, const float *pos4, const float *vel4, const float *mass,
                         double eps2, double out[8], int threads) {
    set_threads(threads);
    double ke = 0, pe = 0, px = 0, py = 0, pz = 0, lx = 0, ly = 0, lz = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : ke, pe, px, py, pz, lx, ly, lz)
    for (int64_t i = 0; i < n; ++i) {
        const double m = mass[i];
        const double x = pos4[4 * i], y = pos4[4 * i + 1], z = pos4[4 * i + 2];
        const double vx = vel4[4 * i], vy = vel4[4 * i + 1], vz = vel4[4 * i + 2];
        ke += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        px += m * vx; py += m * vy; pz += m * vz;
        lx += m * (y * vz - z * vy); ly += m * (z * vx - x * vz); lz += m * (x * vy - y * vx);
        double p = 0.0;
        for (int64_t j = i + 1; j < n; ++j) {
            const double dx = pos4[4 * j] - x, dy = pos4[4 * j + 1] - y, dz = pos4[4 * j + 2] - z;
            p += (double)mass[j] / sqrt(dx * dx + dy * dy + dz * dz + eps2);
        }
        pe -= m * p;
    }
    out[0] = ke; out[1] = pe; out[2] = px; out[3] = py; out[4] = pz; out[5] = lx; out[6] = ly; out[7] = lz;
}
