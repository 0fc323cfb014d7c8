/* CPU oracle, integer/bit-exact part: 63-bit Morton keys and a stable sort.
 *
 * TEST INFRASTRUCTURE ONLY (see nbody_oracle.h). Built with strict IEEE
 * arithmetic (no -ffast-math, no FMA contraction): the GPU keys must equal
 * these bit for bit.
 */
#include "nbody_oracle.h"

#include <stdlib.h>
#include <string.h>

/* ---- 63-bit Morton keys --------------------------------------------------
 * Restates src/shaders/ComputeShaders/morton.glsl with 21 bits per axis:
 *   extent = max(bmax - bmin, 1e-6)                          (:69-70)
 *   norm   = clamp((p - bmin) / extent, 0, 1)                 (:73-74)
 *   q      = uint(min(max(norm * 2^21, 0), 2^21 - 1))         (:49-51)
 *   key    = expand(qx) << 2 | expand(qy) << 1 | expand(qz)   (:63, x highest)
 * Every step is one correctly rounded IEEE-754 binary32 operation (sub, div,
 * compare, multiply by a power of two, compare, truncate); this file is
 * compiled WITHOUT -ffast-math and with -ffp-contract=off so that the compiler
 * keeps exactly these operations. */
static inline uint64_t expand21(uint64_t v) {
    v &= 0x1FFFFFull;
    v = (v | (v << 32)) & 0x001F00000000FFFFull;
    v = (v | (v << 16)) & 0x001F0000FF0000FFull;
    v = (v | (v << 8)) & 0x100F00F00F00F00Full;
    v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

static inline uint32_t quantize21(float p, float lo, float hi) {
    float ext = hi - lo;
    if (!(ext > 1e-6f)) ext = 1e-6f;   /* max(extent, 1e-6) */
    float t = (p - lo) / ext;
    if (t < 0.f) t = 0.f;                /* clamp(norm, 0, 1) */
    if (t > 1.f) t = 1.f;
    float g = t * 2097152.0f;            /* exact: power of two */
    if (g > 2097151.0f) g = 2097151.0f;
    return (uint32_t)g;                  /* truncation toward zero */
}

uint64_t orc_morton63_key(float px, float py, float pz, const float bmin[3], const float bmax[3]) {
    const uint64_t qx = quantize21(px, bmin[0], bmax[0]);
    const uint64_t qy = quantize21(py, bmin[1], bmax[1]);
    const uint64_t qz = quantize21(pz, bmin[2], bmax[2]);
    return (expand21(qx) << 2) | (expand21(qy) << 1) | expand21(qz);
}

void orc_morton63(int64_t n, const float *pos4, const float bmin[3], const float bmax[3], uint64_t *keys) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) keys[i] = orc_morton63_key(pos4[4 * i], pos4[4 * i + 1], pos4[4 * i + 2], bmin, bmax);
}

/* ---- octree-descent keys ------------------------------------------------
 * The reference's own child selection, Octree::getNextNode with the child
 * boxes of Octree::subdivide (src/Octree/Octree.cpp:148-231), applied 21 times
 * from the root box: per level and axis, centre = min + (max - min) / 2 and the
 * body goes to the upper half unless pos < centre; key bit 1 = upper half, x
 * highest in each triple. */
uint64_t orc_octree_key(float px, float py, float pz, const float bmin[3], const float bmax[3]) {
    float mn[3] = {bmin[0], bmin[1], bmin[2]};
    float mx[3] = {bmax[0], bmax[1], bmax[2]};
    const float p[3] = {px, py, pz};
    uint64_t key = 0;
    for (int l = 0; l < 21; ++l) {
        uint64_t digit = 0;
        for (int a = 0; a < 3; ++a) {
            const float w = mx[a] - mn[a];
            const float c = mn[a] + w / 2.f;
            const int upper = !(p[a] < c);
            if (upper) mn[a] = c; else mx[a] = c;
            digit |= (uint64_t)upper << (2 - a);
        }
        key = (key << 3) | digit;
    }
    return key;
}

void orc_octree_keys(int64_t n, const float *pos4, const float bmin[3], const float bmax[3], uint64_t *keys) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) keys[i] = orc_octree_key(pos4[4 * i], pos4[4 * i + 1], pos4[4 * i + 2], bmin, bmax);
}

/* ---- stable sort: LSD radix, 8 bits per pass (stable by construction) ---- */
int orc_sort_stable(int64_t n, const uint64_t *keys, uint64_t *keys_sorted, uint32_t *perm) {
    if (n < 0) return ORC_ERR_ARG;
    uint64_t *ka = malloc(sizeof(uint64_t) * (size_t)(n ? n : 1));
    uint64_t *kb = malloc(sizeof(uint64_t) * (size_t)(n ? n : 1));
    uint32_t *pa = malloc(sizeof(uint32_t) * (size_t)(n ? n : 1));
    uint32_t *pb = malloc(sizeof(uint32_t) * (size_t)(n ? n : 1));
    if (!ka || !kb || !pa || !pb) { free(ka); free(kb); free(pa); free(pb); return ORC_ERR_NOMEM; }
    for (int64_t i = 0; i < n; ++i) { ka[i] = keys[i]; pa[i] = (uint32_t)i; }
    for (int pass = 0; pass < 8; ++pass) {
        const int sh = 8 * pass;
        int64_t cnt[257];
        memset(cnt, 0, sizeof(cnt));
        for (int64_t i = 0; i < n; ++i) cnt[((ka[i] >> sh) & 0xFF) + 1]++;
        for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
        for (int64_t i = 0; i < n; ++i) {
            const int d = (int)((ka[i] >> sh) & 0xFF);
            const int64_t o = cnt[d]++;
            kb[o] = ka[i];
            pb[o] = pa[i];
        }
        uint64_t *tk = ka; ka = kb; kb = tk;
        uint32_t *tp = pa; pa = pb; pb = tp;
    }
    for (int64_t i = 0; i < n; ++i) {
        if (keys_sorted) keys_sorted[i] = ka[i];
        perm[i] = pa[i];
    }
    free(ka); free(kb); free(pa); free(pb);
    return ORC_OK;
}

