// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror and Shaw, "Parallel
// random numbers: as easy as 1, 2, 3", SC'11), written from the published
// description: 10 rounds of two 32x32->64 multiplications with the round key
// bumped by the Weyl constants between rounds.  Host and device share this code,
// so the thermostat noise of a step is a pure function of (seed, step, atom) and
// the CPU restatement can reproduce it.
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define ATM_HD __host__ __device__ __forceinline__
#else
#define ATM_HD inline
#endif

namespace atm {

struct U32x4 {
    uint32_t v[4];
};

ATM_HD void philox_mulhilo(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
}

ATM_HD U32x4 philox4x32_10(U32x4 c, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    for (int r = 0; r < 10; r++) {
        uint32_t hi0, lo0, hi1, lo1;
        philox_mulhilo(M0, c.v[0], &hi0, &lo0);
        philox_mulhilo(M1, c.v[2], &hi1, &lo1);
        U32x4 n;
        n.v[0] = hi1 ^ c.v[1] ^ k0;
        n.v[1] = lo1;
        n.v[2] = hi0 ^ c.v[3] ^ k1;
        n.v[3] = lo0;
        c = n;
        k0 += W0;
        k1 += W1;
    }
    return c;
}

// Uniform in the open interval (0, 1) from 32 random bits.
ATM_HD double philox_uniform(uint32_t r) { return ((double)r + 0.5) * 2.3283064365386963e-10; }

// Streams of the counter's last word (bit 0; the replica index fills the others).
enum RandomStream : uint32_t { RNG_THERMOSTAT = 0, RNG_VELOCITIES = 1 };

}  // namespace atm
