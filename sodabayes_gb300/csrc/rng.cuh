// rng.cuh — counter-based draws for the SODA sampler (device side).
//
// The reference gives every OpenMP thread its own xoroshiro128+ stream
// (parallelrng.f90:54-149), so a SNP's draws depend on which thread ran it.
// On the GPU each draw is instead keyed by (seed, chain, iteration, slot,
// purpose): Philox4x32-10 (Salmon, Moraes, Dror & Shaw, SC'11) turns that
// counter into 64-bit words, which are mapped to [0,1) exactly like
// rng_int64_to_real64 (parallelrng.f90:242-249).  The distributions below
// restate the reference's transforms:
//   normal         Box-Muller, sine branch, REAL-precision pi (parallelrng.f90:264-277)
//   gamma          Marsaglia & Tsang 2000, boost for shape<1  (parallelrng.f90:294-333)
//   inv. chi^2     1/gamma(dof/2, 2/(dof*scale))               (parallelrng.f90:348-362)
//   Dirichlet      normalised gammas                            (parallelrng.f90:445-455)
#pragma once
#include <stdint.h>
#include "../../include/sodagpu.h"

namespace soda {

// Purposes (third counter word); the CPU oracle uses the same numbering.
enum Purpose : uint32_t {
    P_SNP = 1, P_MU = 2, P_VARA = 3, P_VARE = 4, P_PI = 5, P_RA = 6,
    P_SKIP = 7, P_PERM = 8, P_POWER = 9
};

// parallelrng.f90:20 declares pi as a default REAL literal: float(pi) widened.
#define SODA_REF_PI 3.1415927410125732

// Device error code of a draw that overran its injected-draw tape record.
constexpr int CRNG_TAPE_OVERRUN = 19;

struct CRng {
    uint32_t k0, k1, c0, c1, c2, c3;
    uint32_t o0, o1, o2, o3;
    int have;   // cached outputs of the last block: 2 both halves, 1 the second, 0 none
    // injected draws: the uniforms of this draw site come from a tape record
    // of SODAGPU_TAPE_W values instead of Philox; tover is set on overrun
    const double *tape;
    int tpos;
    int *tover;
};

__host__ __device__ __forceinline__ uint32_t mulhi32(uint32_t a, uint32_t b)
{
#if defined(__CUDA_ARCH__)
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

__host__ __device__ __forceinline__ void philox4x32_10(uint32_t &c0, uint32_t &c1, uint32_t &c2,
                                                       uint32_t &c3, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint32_t lo0 = 0xD2511F53u * c0, hi0 = mulhi32(0xD2511F53u, c0);
        const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = mulhi32(0xCD9E8D57u, c2);
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
}

__host__ __device__ __forceinline__ void crng_init(CRng &s, uint64_t seed, int chain, int iter,
                                                   int slot, int purpose)
{
    s.k0 = (uint32_t)seed;
    s.k1 = (uint32_t)(seed >> 32);
    s.c0 = (uint32_t)iter;
    s.c1 = (uint32_t)slot;
    s.c2 = (uint32_t)purpose;
    s.c3 = (uint32_t)chain << 20;
    s.have = 0;
    s.tape = nullptr;
    s.tpos = 0;
    s.tover = nullptr;
}

__device__ __forceinline__ double crng_tape_next(CRng &s)
{
    double v = 0.5;
    if (s.tpos < SODAGPU_TAPE_W) v = s.tape[s.tpos];
    else if (s.tover) *s.tover = CRNG_TAPE_OVERRUN;
    ++s.tpos;
    return v;
}

// Computes the first Philox block of a draw site ahead of its first use (the
// counters do not depend on the data, so a kernel can do this before waiting
// for the kernel that produces them): crng_u64 then returns the same values.
__host__ __device__ __forceinline__ void crng_warm(CRng &s)
{
    if (s.have != 0 || s.tape) return;
    uint32_t a = s.c0, b = s.c1, c = s.c2, d = s.c3;
    philox4x32_10(a, b, c, d, s.k0, s.k1);
    s.c3++;
    s.o0 = a;
    s.o1 = b;
    s.o2 = c;
    s.o3 = d;
    s.have = 2;
}

__host__ __device__ __forceinline__ uint64_t crng_u64(CRng &s)
{
    if (s.have == 2) {
        s.have = 1;
        return ((uint64_t)s.o1 << 32) | s.o0;
    }
    if (s.have == 0) {
        uint32_t a = s.c0, b = s.c1, c = s.c2, d = s.c3;
        philox4x32_10(a, b, c, d, s.k0, s.k1);
        s.c3++;
        s.o2 = c;
        s.o3 = d;
        s.have = 1;
        return ((uint64_t)b << 32) | a;
    }
    s.have = 0;
    return ((uint64_t)s.o3 << 32) | s.o2;
}

__host__ __device__ __forceinline__ double crng_unit(CRng &s)
{
#if defined(__CUDA_ARCH__)
    if (s.tape) return crng_tape_next(s);
#endif
    const uint64_t bits = 0x3FF0000000000000ULL | (crng_u64(s) >> 12);
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)bits) - 1.0;
#else
    double d;
    __builtin_memcpy(&d, &bits, sizeof d);
    return d - 1.0;
#endif
}

// rand_normal (parallelrng.f90:264-277)
__device__ __forceinline__ double d_rnorm(double mean, double sd, CRng &s)
{
    if (sd <= 0.0) return mean;
    const double u1 = crng_unit(s), u2 = crng_unit(s);
    const double rr = sqrt(-2.0 * log(u1));
    const double th = 2.0 * SODA_REF_PI * u2;
    return mean + sd * rr * sin(th);
}

// rand_gamma (parallelrng.f90:294-333).  The rejection loop is bounded; on
// the (practically impossible) exhaustion *err is set and the last candidate
// returned.
__device__ __forceinline__ double d_rgamma(double shape, double scale, CRng &s, int *err)
{
    const bool small = shape < 1.0;
    const double sh = small ? shape + 1.0 : shape;
    const double sc = small ? 1.0 : scale;
    const double d = sh - 1.0 / 3.0;
    const double c = 1.0 / sqrt(9.0 * d);
    double res = d;
    int tries = 0;
    for (;;) {
        double x = d_rnorm(0.0, 1.0, s);
        double v = 1.0 + c * x;
        while (v <= 0.0 && tries < 100000) {
            x = d_rnorm(0.0, 1.0, s);
            v = 1.0 + c * x;
            ++tries;
        }
        v = v * v * v;
        const double u = crng_unit(s);
        const double xsq = x * x;
        res = sc * d * v;
        if ((u < 1.0 - 0.0331 * xsq * xsq) || (log(u) < 0.5 * xsq + d * (1.0 - v + log(v)))) break;
        if (++tries >= 100000) { if (err) *err = 1; break; }
    }
    if (small) {
        // shape < 1: g ~ gamma(shape+1, 1), then scale*g*w**(1/shape)
        const double w = crng_unit(s);
        return scale * res * pow(w, 1.0 / shape);
    }
    return res;
}

// rand_scaled_inverse_chi_square (parallelrng.f90:348-362)
__device__ __forceinline__ double d_rscinvchi2(double dof, double scale, CRng &s, int *err)
{
    const double shape = 0.5 * dof, sc = 0.5 * dof * scale;
    return 1.0 / d_rgamma(shape, 1.0 / sc, s, err);
}

// ---------------------------------------------------------------------------
// FP32 transforms for the reduced-precision sweeps (same counter streams).
// Uniforms take the top 24 bits of each word, offset by half a unit so they
// lie strictly inside (0,1): log(u) is always finite.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float crng_unit_f(CRng &s)
{
    if (s.tape) return (float)crng_tape_next(s);
    return ((float)(uint32_t)(crng_u64(s) >> 40) + 0.5f) * 5.9604644775390625e-8f;
}

__device__ __forceinline__ float d_rnorm_f(float mean, float sd, CRng &s)
{
    if (sd <= 0.0f) return mean;
    const float u1 = crng_unit_f(s), u2 = crng_unit_f(s);
    const float rr = sqrtf(-2.0f * logf(u1));
    const float th = 6.2831854820251465f * u2;
    return mean + sd * rr * sinf(th);
}

__device__ __forceinline__ float d_rgamma_f(float shape, float scale, CRng &s, int *err)
{
    const bool small = shape < 1.0f;
    const float sh = small ? shape + 1.0f : shape;
    const float sc = small ? 1.0f : scale;
    const float d = sh - 1.0f / 3.0f;
    const float c = 1.0f / sqrtf(9.0f * d);
    float res = d;
    int tries = 0;
    for (;;) {
        float x = d_rnorm_f(0.0f, 1.0f, s);
        float v = 1.0f + c * x;
        while (v <= 0.0f && tries < 100000) {
            x = d_rnorm_f(0.0f, 1.0f, s);
            v = 1.0f + c * x;
            ++tries;
        }
        v = v * v * v;
        const float u = crng_unit_f(s);
        const float xsq = x * x;
        res = sc * d * v;
        if ((u < 1.0f - 0.0331f * xsq * xsq) || (logf(u) < 0.5f * xsq + d * (1.0f - v + logf(v)))) break;
        if (++tries >= 100000) { if (err) *err = 1; break; }
    }
    if (small) {
        const float w = crng_unit_f(s);
        return scale * res * powf(w, 1.0f / shape);
    }
    return res;
}

__device__ __forceinline__ float d_rscinvchi2_f(float dof, float scale, CRng &s, int *err)
{
    const float shape = 0.5f * dof, sc = 0.5f * dof * scale;
    return 1.0f / d_rgamma_f(shape, 1.0f / sc, s, err);
}

}  // namespace soda
