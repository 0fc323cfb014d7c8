// Seeded initial conditions generated on the device, straight into the
// resident state (no host generation and no host-to-device copy).
//
// The reference's initialisers (src/ParticleSystemInitializer/*) draw from
// std::random_device or the clock, so their runs cannot be repeated; these
// kernels restate their shapes with a counter-based generator: draw k of body
// i under seed s is a fixed function of (s, i, k), so the result does not
// depend on the launch shape. Velocity w and acceleration are zero.
#include <cuda_runtime.h>

#include "common.cuh"
#include "init.h"

namespace nbody {

namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    // splitmix64 (Steele, Lea, Flood 2014) output function
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Uniform on [0, 1) with 24 random bits (exactly representable in FP32).
__device__ __forceinline__ float u01(uint64_t seed, int64_t i, uint32_t k) {
    const uint64_t h = mix64(seed ^ mix64(static_cast<uint64_t>(i) * 0xD1B54A32D192ED03ull + k));
    return static_cast<float>(h >> 40) * (1.0f / 16777216.0f);
}

// Uniform on [a, b), rounded once per operation.
__device__ __forceinline__ float uab(uint64_t seed, int64_t i, uint32_t k, float a, float b) {
    return __fadd_rn(a, __fmul_rn(__fsub_rn(b, a), u01(seed, i, k)));
}

// Standard normal by Box-Muller from draws k, k + 1.
__device__ __forceinline__ float normal01(uint64_t seed, int64_t i, uint32_t k) {
    const float u1 = 1.f - u01(seed, i, k);  // (0, 1]
    const float u2 = u01(seed, i, k + 1);
    return sqrtf(-2.f * logf(u1)) * cospif(2.f * u2);
}

// Isotropic unit vector from draws k, k + 1.
__device__ __forceinline__ float3 unit_vector(uint64_t seed, int64_t i, uint32_t k) {
    const float z = 2.f * u01(seed, i, k) - 1.f;
    const float r = sqrtf(fmaxf(0.f, 1.f - z * z));
    float s, c;
    sincospif(2.f * u01(seed, i, k + 1), &s, &c);
    return make_float3(r * c, r * s, z);
}

__device__ __forceinline__ float norm3(float3 v) { return sqrtf(v.x * v.x + v.y * v.y + v.z * v.z); }
__device__ __forceinline__ float3 scale3(float3 v, float s) { return make_float3(s * v.x, s * v.y, s * v.z); }
__device__ __forceinline__ float3 add3(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }

struct Body {
    float3 x, v;
    float m;
};

// ParticleSystemCubeInitializer.cpp:15-27: every coordinate uniform on [0, W.x)
// (the x extent on all axes, as in the reference), velocity uniform on
// [-|W|/20, |W|/20) per axis, mass (volume / n) * 1.2 * U[0.8, 1.3). W.z = 0
// gives a plane.
__device__ Body cube(uint64_t s, int64_t i, int64_t n, float3 W) {
    const bool flat = W.z == 0.f;
    const float l = norm3(W) / 20.f;
    Body b;
    b.x = make_float3(uab(s, i, 0, 0.f, W.x), uab(s, i, 1, 0.f, W.x), flat ? 0.f : uab(s, i, 2, 0.f, W.x));
    b.v = make_float3(uab(s, i, 3, -l, l), uab(s, i, 4, -l, l), flat ? 0.f : uab(s, i, 5, -l, l));
    b.m = (W.x * W.y * W.z / static_cast<float>(n)) * 1.2f * uab(s, i, 6, 0.8f, 1.3f);
    return b;
}

// ParticleSystemGalaxyInitializer.cpp:46-90 (its first, fixed-shape branch):
// radius U[0, W.x), angle N(0, 50 pi) * 2 pi, height U[0.1, W.z / 5) above the
// mid-plane through the world centre; mass (volume / n) * 0.7 inside the bulge
// (radius < W.x / 10), else * 0.5; tangential speed |W| / 4 plus, inside
// W.x / 2, the arm term |W| / 4 * (r / (W.x / 2)) * cos(6 (atan2 - angle))
// along -radial.
__device__ Body galaxy(uint64_t s, int64_t i, int64_t n, float3 W) {
    const float3 C = scale3(W, 0.5f);
    const float volume = W.x * W.y * W.z;
    const float L = norm3(W) / 4.f;
    const float r = uab(s, i, 0, 0.f, W.x);
    const float theta = normal01(s, i, 1) * (3.1415f * 50.f) * (2.f * 3.14159265f);
    const float h = W.z == 0.f ? 0.f : uab(s, i, 3, 0.1f, W.z / 5.f);
    float sn, cs;
    sincosf(theta, &sn, &cs);
    Body b;
    b.x = add3(C, make_float3(r * cs, r * sn, h));
    b.m = (volume / static_cast<float>(n)) * (r < W.x / 10.f ? 0.7f : 0.5f);
    b.v = make_float3(-L * sn, L * cs, 0.f);
    const float arm_r = W.x / 2.f;
    if (r < arm_r) {
        const float ang = atan2f(b.x.y - C.y, b.x.x - C.x);
        const float mag = L * (r / arm_r) * cosf(6.f * (ang - theta));
        b.v = add3(b.v, make_float3(-mag * cs, -mag * sn, 0.f));
    }
    return b;
}

// ParticleSystemSphere.cpp:20-95: on the sphere of radius |W|/3 about the world
// centre; speed U[0.5, 1.5) * |W| / 15 outward (pattern 0), inward (1) or
// along axis x r with axis = normalize(0.2, 1, -0.1) (2); mass
// (volume / n) * 0.5 * U[0.7, 1.3). The reference picks the pattern at random
// per run; here it is a parameter.
__device__ Body sphere(uint64_t s, int64_t i, int64_t n, float3 W, int pattern) {
    const float R = norm3(W) / 3.f;
    const float3 u = unit_vector(s, i, 0);
    Body b;
    b.x = add3(scale3(W, 0.5f), scale3(u, R));
    b.m = (W.x * W.y * W.z / static_cast<float>(n)) * 0.5f * uab(s, i, 2, 0.7f, 1.3f);
    const float speed = (norm3(W) / 15.f) * uab(s, i, 3, 0.5f, 1.5f);
    if (pattern == 2) {
        const float al = sqrtf(0.2f * 0.2f + 1.f + 0.1f * 0.1f);
        const float3 ax = make_float3(0.2f / al, 1.f / al, -0.1f / al);
        float3 t = make_float3(ax.y * u.z - ax.z * u.y, ax.z * u.x - ax.x * u.z, ax.x * u.y - ax.y * u.x);
        const float tl = norm3(t);
        // Along the axis the reference falls back to a small random direction.
        b.v = tl > 1e-6f ? scale3(t, speed / tl) : scale3(unit_vector(s, i, 4), 0.1f * speed);
    } else {
        b.v = scale3(u, pattern == 1 ? -speed : speed);
    }
    return b;
}

// ParticleSystemBall.cpp:19-75: uniform in the ball of radius |W|/3 about the
// centre (rejection from the cube, a bounded number of tries), nudged by
// U[-1, 1) * 5% of the radius per axis; velocity U[-1, 1) * |W| / 1000 per
// axis; mass min + (max - min) u^2 with avg = volume / n, min = avg / 2,
// max = 5 avg. W.z = 0 gives a disc.
__device__ Body ball(uint64_t s, int64_t i, int64_t n, float3 W) {
    const bool flat = W.z == 0.f;
    const float R = norm3(W) / 3.f;
    float3 p = make_float3(0.f, 0.f, 0.f);
    for (uint32_t t = 0; t < 64; ++t) {
        const uint32_t k = 16 + 3 * t;
        const float3 q = make_float3(uab(s, i, k, -1.f, 1.f) * R, uab(s, i, k + 1, -1.f, 1.f) * R,
                                     flat ? 0.f : uab(s, i, k + 2, -1.f, 1.f) * R);
        if (q.x * q.x + q.y * q.y + q.z * q.z <= R * R) {
            p = q;
            break;
        }
    }
    const float pert = 0.05f * R;
    p = add3(p, make_float3(uab(s, i, 0, -1.f, 1.f) * pert, uab(s, i, 1, -1.f, 1.f) * pert,
                            flat ? 0.f : uab(s, i, 2, -1.f, 1.f) * pert));
    const float vs = norm3(W) * 0.001f;
    Body b;
    b.x = add3(scale3(W, 0.5f), p);
    b.v = make_float3(uab(s, i, 3, -1.f, 1.f) * vs, uab(s, i, 4, -1.f, 1.f) * vs,
                      flat ? 0.f : uab(s, i, 5, -1.f, 1.f) * vs);
    const float avg = W.x * W.y * W.z / static_cast<float>(n);
    const float lo = avg * 0.5f, hi = avg * 5.f;
    const float u = u01(s, i, 6);
    b.m = lo + (hi - lo) * (u * u);
    return b;
}

// ParticleSystemCubeSurface.cpp:15-50: a face chosen uniformly, the two free
// coordinates U[-W.x/2, W.x/2), then shifted by W/2; velocity and mass as for
// the cube.
__device__ Body cube_surface(uint64_t s, int64_t i, int64_t n, float3 W) {
    const int face = min(5, static_cast<int>(u01(s, i, 0) * 6.f));
    const float a = uab(s, i, 1, -W.x / 2.f, W.x / 2.f), c = uab(s, i, 2, -W.x / 2.f, W.x / 2.f);
    float3 q;
    switch (face) {
        case 0: q = make_float3(-W.x / 2.f, a, c); break;
        case 1: q = make_float3(W.x / 2.f, a, c); break;
        case 2: q = make_float3(a, -W.y / 2.f, c); break;
        case 3: q = make_float3(a, W.y / 2.f, c); break;
        case 4: q = make_float3(a, c, -W.z / 2.f); break;
        default: q = make_float3(a, c, W.z / 2.f); break;
    }
    const bool flat = W.z == 0.f;
    const float l = norm3(W) / 20.f;
    Body b;
    b.x = add3(q, scale3(W, 0.5f));
    b.v = make_float3(uab(s, i, 3, -l, l), uab(s, i, 4, -l, l), flat ? 0.f : uab(s, i, 5, -l, l));
    b.m = (W.x * W.y * W.z / static_cast<float>(n)) * 1.2f * uab(s, i, 6, 0.8f, 1.3f);
    return b;
}

// Uniform ball about the origin at rest: p[0] radius, p[1], p[2] mass range.
__device__ Body uniform_ball(uint64_t s, int64_t i, const float *p) {
    Body b;
    b.x = scale3(unit_vector(s, i, 0), p[0] * cbrtf(u01(s, i, 2)));
    b.v = make_float3(0.f, 0.f, 0.f);
    b.m = uab(s, i, 3, p[1], p[2]);
    return b;
}

// Equal-mass Plummer sphere, G = 1: p[0] scale radius a, p[1] body mass,
// p[2] truncation radius / a. r = a / sqrt(u^(-2/3) - 1), redrawn beyond the
// truncation; speed q v_esc(r) with q drawn from q^2 (1 - q^2)^3.5 by rejection
// (Aarseth, Henon, Wielen 1974); isotropic directions. Both rejection loops are
// bounded; the acceptance rates are above 0.99 and about 0.5.
__device__ Body plummer(uint64_t s, int64_t i, int64_t n, const float *p) {
    const float a = p[0], mb = p[1], rmax = p[2] * p[0];
    float r = rmax;
    for (uint32_t k = 0; k < 64; ++k) {
        const float u = fmaxf(u01(s, i, 16 + k), 1e-7f);
        const float rr = a * rsqrtf(powf(u, -2.f / 3.f) - 1.f);
        if (rr <= rmax) {
            r = rr;
            break;
        }
    }
    float q = 0.f;
    for (uint32_t k = 0; k < 256; ++k) {
        const float x = u01(s, i, 80 + 2 * k);
        const float y = 0.1f * u01(s, i, 81 + 2 * k);
        q = x;
        if (y < x * x * powf(1.f - x * x, 3.5f)) break;
    }
    const float vesc = sqrtf(2.f * mb * static_cast<float>(n) * rsqrtf(r * r + a * a));
    Body b;
    b.x = scale3(unit_vector(s, i, 0), r);
    b.v = scale3(unit_vector(s, i, 2), q * vesc);
    b.m = mb;
    return b;
}

// Two exponential discs, each with a central point mass first: body 0 and body
// n/2 are the centres. p[0] scale length Rd, p[1] sech^2 scale height, p[2]
// central mass, p[3] separation along x, p[4] relative speed along y, p[5]
// inclination of the second disc about x in degrees, p[6] softening eps^2 used
// for the circular speed, p[7] star mass. Radii R = -Rd ln(u1 u2) (surface
// density ~ exp(-R/Rd)); circular speed from the central mass plus the stars'
// expected enclosed mass m (n/2 - 1) (1 - (1 + R/Rd) exp(-R/Rd)), softened.
__device__ Body two_discs(uint64_t s, int64_t i, int64_t n, const float *p) {
    const int64_t half = n / 2;
    const int disc = i < half ? 0 : 1;
    const int64_t j = i - disc * half;
    const float Rd = p[0], hz = p[1], Mc = p[2], ms = p[7];
    float3 x = make_float3(0.f, 0.f, 0.f), v = make_float3(0.f, 0.f, 0.f);
    float m = Mc;
    if (j > 0) {
        const float u1 = 1.f - u01(s, i, 0), u2 = 1.f - u01(s, i, 1);
        const float R = -Rd * logf(u1 * u2);
        float sn, cs;
        sincospif(2.f * u01(s, i, 2), &sn, &cs);
        const float t = fminf(fmaxf(2.f * u01(s, i, 3) - 1.f, -0.999999f), 0.999999f);
        const float z = hz * atanhf(t);
        const float y = R / Rd;
        const float enc = Mc + ms * static_cast<float>(half - 1) * (1.f - (1.f + y) * expf(-y));
        const float d2 = R * R + p[6];
        const float vc = sqrtf(enc * R * R / (d2 * sqrtf(d2)));
        x = make_float3(R * cs, R * sn, z);
        v = make_float3(-vc * sn, vc * cs, 0.f);
        m = ms;
    }
    if (disc == 1) {
        float si, ci;
        sincospif(p[5] / 180.f, &si, &ci);
        x = make_float3(x.x, ci * x.y - si * x.z, si * x.y + ci * x.z);
        v = make_float3(v.x, ci * v.y - si * v.z, si * v.y + ci * v.z);
    }
    const float sign = disc == 0 ? -1.f : 1.f;
    x.x += sign * p[3] / 2.f;
    v.y += sign * p[4] / 2.f;
    Body b;
    b.x = x;
    b.v = v;
    b.m = m;
    return b;
}

__global__ void init_kernel(int kind, uint64_t seed, int64_t n, InitParams prm, float4 *__restrict__ pos,
                            float4 *__restrict__ vel, float4 *__restrict__ acc) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 W = make_float3(prm.p[0], prm.p[1], prm.p[2]);
    Body b;
    switch (kind) {
        case NBODY_INIT_CUBE: b = cube(seed, i, n, W); break;
        case NBODY_INIT_GALAXY: b = galaxy(seed, i, n, W); break;
        case NBODY_INIT_SPHERE: b = sphere(seed, i, n, W, static_cast<int>(prm.p[3])); break;
        case NBODY_INIT_BALL: b = ball(seed, i, n, W); break;
        case NBODY_INIT_CUBE_SURFACE: b = cube_surface(seed, i, n, W); break;
        case NBODY_INIT_UNIFORM_BALL: b = uniform_ball(seed, i, prm.p); break;
        case NBODY_INIT_TWO_DISCS: b = two_discs(seed, i, n, prm.p); break;
        default: b = plummer(seed, i, n, prm.p); break;
    }
    pos[i] = make_float4(b.x.x, b.x.y, b.x.z, b.m);
    vel[i] = make_float4(b.v.x, b.v.y, b.v.z, 0.f);
    acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

}  // namespace

bool init_kind_valid(int kind) {
    switch (kind) {
        case NBODY_INIT_CUBE:
        case NBODY_INIT_GALAXY:
        case NBODY_INIT_SPHERE:
        case NBODY_INIT_BALL:
        case NBODY_INIT_CUBE_SURFACE:
        case NBODY_INIT_PLUMMER:
        case NBODY_INIT_UNIFORM_BALL:
        case NBODY_INIT_TWO_DISCS: return true;
        default: return false;
    }
}

InitParams init_defaults(int kind) {
    InitParams p{};
    switch (kind) {
        case NBODY_INIT_PLUMMER: p = {{100.f, 1.f, 20.f}}; break;
        case NBODY_INIT_UNIFORM_BALL: p = {{100.f, 1.f, 10.f}}; break;
        case NBODY_INIT_TWO_DISCS: p = {{200.f, 20.f, 1e6f, 2000.f, 50.f, 30.f, 40.f, 1.f}}; break;
        default: p = {{5.f, 5.f, 5.f, 0.f}}; break;  // the reference's world, glm::vec3(5.f)
    }
    return p;
}

cudaError_t init_state(int kind, uint64_t seed, int64_t n, const InitParams &prm, float4 *pos, float4 *vel,
                       float4 *acc, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const unsigned blocks = static_cast<unsigned>((n + 255) / 256);
    init_kernel<<<blocks, 256, 0, st>>>(kind, seed, n, prm, pos, vel, acc);
    return cudaGetLastError();
}

}  // namespace nbody
