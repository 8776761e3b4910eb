/*
 * cd_noise.h -- fluctuation noise drawn from a counter-based generator,
 * shared by the device kernels and the CPU oracle (same source, same bits).
 *
 * Generator: Philox4x32-10 (J. K. Salmon, M. A. Moraes, R. O. Dror and
 * D. E. Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC11, 2011):
 * a 4 x 32-bit counter and a 2 x 32-bit key; ten rounds of two 32 x 32 ->
 * 64-bit multiplications (multipliers 0xD2511F53, 0xCD9E8D57) whose high
 * and low halves are permuted and xored with the key, the key bumped by the
 * Weyl constants 0x9E3779B9, 0xBB67AE85 between rounds.  Counter-based: the
 * value for (seed, step, agent, draw) needs no state, so every agent draws
 * independently on any thread, in any order, inside CUDA graphs.
 *
 * Distribution (core/motion/fluctuation.py:14-62, core/rand.py:8-32):
 *   force  = mass * (std_rand_force * xi) * (cos phi, sin phi),
 *            phi ~ U(0, 2 pi), xi ~ N(0, 1) truncated to [0, 3];
 *   torque = inertia_rot * (std_rand_torque * eta), eta ~ N(0, 1) truncated
 *            to [-3, 3].
 * Uniforms take 53 bits from two words.  Normals come from the Box-Muller
 * transform, r = sqrt(-2 log(1 - u1)), theta = 2 pi u2 (both of a pair are
 * used); a truncated normal is the first of them inside the interval
 * ([0, 3] takes |z|, since the half-normal truncated to [0, 3] is N(0, 1)
 * truncated to [0, 3]).  Each draw makes at most 8 generator calls (16
 * normals); all 16 fall outside with probability 0.0027^16 < 1e-40, and the
 * draw then returns 0.
 */
#ifndef CD_NOISE_H
#define CD_NOISE_H

#include "cd_math.h"

CDM_FN void cdn_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2],
                              uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Uniform double in [0, 1) with 53 random bits. */
CDM_FN double cdn_u53(uint32_t hi, uint32_t lo) {
    return ((double)(hi >> 5) * 67108864.0 + (double)(lo >> 6)) * 0x1.0p-53;
}

#define CDN_TWO_PI 0x1.921fb54442d18p+2      /* 2 pi rounded */
#define CDN_TRIES 8

/* Generator output for (seed; step, agent, word3): word3 = stream << 8 | try. */
CDM_FN void cdn_draw(uint64_t seed, uint64_t step, uint32_t agent, uint32_t word3,
                     uint32_t out[4]) {
    const uint32_t ctr[4] = {(uint32_t)step, (uint32_t)(step >> 32), agent, word3};
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    cdn_philox4x32_10(ctr, key, out);
}

/* Standard normal truncated to [0, 3] (half) or [-3, 3], from stream `stream`. */
CDM_FN double cdn_truncnorm3(uint64_t seed, uint64_t step, uint32_t agent, uint32_t stream,
                             int half) {
    for (uint32_t t = 0; t < CDN_TRIES; ++t) {
        uint32_t w[4];
        cdn_draw(seed, step, agent, (stream << 8) | (t + 1), w);
        const double u1 = cdn_u53(w[0], w[1]), u2 = cdn_u53(w[2], w[3]);
        const double r = sqrt(-2.0 * cdm_log(1.0 - u1));
        double sn, cs;
        cdm_sincos(CDN_TWO_PI * u2, &sn, &cs);
        double z0 = r * cs, z1 = r * sn;
        if (half) { z0 = fabs(z0); z1 = fabs(z1); }
        if (z0 >= -3.0 && z0 <= 3.0) return z0;
        if (z1 >= -3.0 && z1 <= 3.0) return z1;
    }
    return 0.0;
}

/* Fluctuation of one agent: force (fx, fy) and, for ThreeCircle, torque. */
CDM_FN void cdn_fluctuation(uint64_t seed, uint64_t step, uint32_t agent, double mass,
                            double std_force, double inertia, double std_torque, int three,
                            double *fx, double *fy, double *tq) {
    uint32_t w[4];
    cdn_draw(seed, step, agent, 0u, w);
    const double phi = CDN_TWO_PI * cdn_u53(w[0], w[1]);
    double sn, cs;
    cdm_sincos(phi, &sn, &cs);
    const double magnitude = 0.0 + std_force * cdn_truncnorm3(seed, step, agent, 1u, 1);
    const double mm = mass * magnitude;
    *fx = mm * cs;
    *fy = mm * sn;
    *tq = three ? inertia * (0.0 + std_torque * cdn_truncnorm3(seed, step, agent, 2u, 0)) : 0.0;
}

#endif
