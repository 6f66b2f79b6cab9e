// Hand-written 3D FFTs of the PME grids with the reciprocal-space convolution
// fused in, sm_103a.  They replace a library R2C / convolution / C2R sequence
// with three kernels, each of which reads and writes every grid once:
//
//   k_fft_zy      one CTA per (grid, x-plane): the plane's real z-rows, two at a
//                 time as one complex row (a + ib), are transformed along z and
//                 split into the half spectra of the two rows; the plane is then
//                 transformed along y and written to the spectrum;
//   k_fft_x_conv  one CTA per (replica, ky, kz chunk): both grids of the replica
//                 are transformed along x, multiplied by the influence function
//                 G(m) (energies summed in FP64), transformed back along x;
//   k_ifft_yz     one CTA per (grid, x-plane): the inverse of k_fft_zy (y, then the
//                 half spectra of two rows recombined and transformed along z).
//
// Every 1D transform is a mixed-radix Stockham FFT in shared memory (no bit
// reversal: each stage reads with stride N/R and writes its R outputs in sorted
// order), radices 8, 4, 2, 3, 5, 7 with dedicated butterflies and a direct DFT
// stage for any other prime factor.  Twiddles come from tables computed in FP64
// on the host.  Transforms are unnormalised (the convolution's prefactor carries
// the scale), the layout of the spectrum is [y][x][z/2 + 1].
//
// Grid 0 of a replica holds state 1's charges; grid 1 holds the structure-factor
// update of the moving atoms, dQ = Q(moving atoms at x + d) - Q(at x).  The
// convolution returns phi1 = G * Q1 and either G * dQ (difference mode: the
// potential of the moved charges) or G * (Q1 + dQ) = phi2 (two-state mode: state
// 2's potential); the energies are E_rec1 = 1/2 sum G |Q1|^2 and
// E_rec2 - E_rec1 = sum G [Re(conj(Q1) dQ) + 1/2 |dQ|^2], so that u's reciprocal
// part is summed directly rather than as a difference of two totals.
#include <algorithm>
#include <cmath>
#include <vector>

#include "kernels.cuh"

namespace atm {

constexpr int kFftThreads = 256;

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiplication by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ float2 rot(float2 a) {
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}
template <bool INV>
__device__ __forceinline__ float2 twid(const float2* tw, int t) {
    const float2 w = tw[t];
    return INV ? make_float2(w.x, -w.y) : w;
}

// Asynchronous global -> shared copies (cp.async): every load of a CTA's input
// is in flight at once, and none occupies registers while it is.
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
// Waits for this thread's copies; a __syncthreads() then publishes them to the CTA.
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// Compensated FP32 sum (Knuth's TwoSum): s + c carries the exact sum of the
// terms up to a relative error of order 2^-48, with FP32 instructions only (the
// FP64 pipe of this part is narrow).
__device__ __forceinline__ void two_sum_add(float& s, float& c, float x) {
    const float t = s + x;
    const float bp = t - s;
    c += (s - (t - bp)) + (x - bp);
    s = t;
}

// Small DFTs in registers, sign -1 (forward) or +1 (INV).
template <bool INV>
__device__ __forceinline__ void dft2(float2* v) {
    const float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}
template <bool INV>
__device__ __forceinline__ void dft4(float2* v) {
    const float2 s0 = cadd(v[0], v[2]), d0 = csub(v[0], v[2]);
    const float2 s1 = cadd(v[1], v[3]), d1 = rot<INV>(csub(v[1], v[3]));
    v[0] = cadd(s0, s1);
    v[2] = csub(s0, s1);
    v[1] = cadd(d0, d1);
    v[3] = csub(d0, d1);
}
template <bool INV>
__device__ __forceinline__ void dft8(float2* v) {
    float2 e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    dft4<INV>(e);
    dft4<INV>(o);
    const float h = 0.70710678118654752f;
    // o[k] *= w8^k, w8 = exp(-+ i pi / 4)
    o[1] = make_float2(h * (o[1].x + (INV ? -o[1].y : o[1].y)), h * (o[1].y + (INV ? o[1].x : -o[1].x)));
    o[2] = rot<INV>(o[2]);
    o[3] = make_float2(h * ((INV ? -o[3].y : o[3].y) - o[3].x), h * ((INV ? o[3].x : -o[3].x) - o[3].y));
#pragma unroll
    for (int k = 0; k < 4; k++) {
        v[k] = cadd(e[k], o[k]);
        v[k + 4] = csub(e[k], o[k]);
    }
}
// Odd radix R (3, 5, 7): X_k = A_k -+ i B_k, X_{R-k} = A_k +- i B_k with
// A_k = x0 + sum_n (x_n + x_{R-n}) cos(2 pi n k / R), B_k = sum_n (x_n - x_{R-n}) sin(2 pi n k / R).
template <int R, bool INV>
__device__ __forceinline__ void dft_odd(float2* v) {
    constexpr int H = (R - 1) / 2;
    float c[R], s[R];
    if (R == 3) {
        c[0] = 1.f; c[1] = c[2] = -0.5f;
        s[0] = 0.f; s[1] = 0.86602540378443865f; s[2] = -s[1];
    } else if (R == 5) {
        c[0] = 1.f; c[1] = c[4] = 0.30901699437494742f; c[2] = c[3] = -0.80901699437494742f;
        s[0] = 0.f; s[1] = 0.95105651629515357f; s[2] = 0.58778525229247313f; s[3] = -s[2]; s[4] = -s[1];
    } else {
        c[0] = 1.f; c[1] = c[6] = 0.62348980185873353f; c[2] = c[5] = -0.22252093395631440f;
        c[3] = c[4] = -0.90096886790241913f;
        s[0] = 0.f; s[1] = 0.78183148246802981f; s[2] = 0.97492791218182361f; s[3] = 0.43388373911755812f;
        s[4] = -s[3]; s[5] = -s[2]; s[6] = -s[1];
    }
    float2 sp[H], sm[H];
#pragma unroll
    for (int n = 1; n <= H; n++) {
        sp[n - 1] = cadd(v[n], v[R - n]);
        sm[n - 1] = csub(v[n], v[R - n]);
    }
    float2 out[R];
    float2 x0 = v[0];
    float2 tot = x0;
#pragma unroll
    for (int n = 0; n < H; n++) tot = cadd(tot, sp[n]);
    out[0] = tot;
#pragma unroll
    for (int k = 1; k <= H; k++) {
        float2 A = x0, B = make_float2(0.f, 0.f);
#pragma unroll
        for (int n = 1; n <= H; n++) {
            const int m = (n * k) % R;
            A.x = fmaf(sp[n - 1].x, c[m], A.x);
            A.y = fmaf(sp[n - 1].y, c[m], A.y);
            B.x = fmaf(sm[n - 1].x, s[m], B.x);
            B.y = fmaf(sm[n - 1].y, s[m], B.y);
        }
        const float2 iB = rot<INV>(B);  // -+ i B
        out[k] = cadd(A, iB);
        out[R - k] = csub(A, iB);
    }
#pragma unroll
    for (int k = 0; k < R; k++) v[k] = out[k];
}

// Division by a divisor 1 <= d < 2^16 fixed for a loop, for non-negative
// w < 2^23: q = umulhi(w, m) with m >= 2^32 / d close to it, so that q is
// floor(w / d) or one more, then corrected.  m is either exact (ceil(2^32 / d),
// from the host's stage plans) or from an FP32 division (within 2^8 of it, q
// then off by at most one either way).  Four integer instructions per division
// instead of a runtime division's sequence.
struct FastDiv {
    unsigned d, m;
    __device__ __forceinline__ explicit FastDiv(int dd)
        : d((unsigned)dd), m(dd > 1 ? (unsigned)(4294967296.0f / (float)dd) : 0u) {}
    __device__ __forceinline__ FastDiv(unsigned dd, unsigned mm) : d(dd), m(mm) {}
    __device__ __forceinline__ unsigned div(unsigned w) const {
        if (d == 1) return w;
        unsigned q = __umulhi(w, m);
        q = q * d > w ? q - 1 : q;
        return (q + 1) * d <= w ? q + 1 : q;
    }
};

// One Stockham stage of radix R (specialised) over nseq sequences of length N
// (element e of sequence q at q * ss + e * es), as planned on the host: Ns the
// product of the earlier radices, nb = N / R butterflies, step = N / (Ns R).
// Butterfly j reads x[j + r nb], twiddles it by w_N^{r k step} (k = j mod Ns) and
// writes its R outputs to (j / Ns) Ns R + k + r Ns.  Work items run
// sequence-fastest: neighbouring threads take neighbouring sequences, whose
// starts the callers space by an odd number of words' pairs (no bank conflicts).
// TW = false: the first stage (Ns = 1), whose twiddles are all 1.
template <int R, bool INV, bool TW>
__device__ __forceinline__ void stage_r(const float2* src, float2* dst, const FftStage& p, const FastDiv& fq,
                                        int ss, int es, const float2* tw) {
    const int nb = p.nb, Ns = TW ? p.Ns : 1, step = p.step;
    const int items = nb * (int)fq.d;
    const FastDiv fns((unsigned)Ns, p.mNs);
    for (int w = threadIdx.x; w < items; w += blockDim.x) {
        const int j = (int)fq.div((unsigned)w), q = w - j * (int)fq.d;
        const int jn = TW ? (int)fns.div((unsigned)j) : j;
        const int k = j - jn * Ns;
        const float2* s = src + q * ss;
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; r++) {
            const float2 x = s[(j + r * nb) * es];
            v[r] = (r == 0 || !TW) ? x : cmul(x, twid<INV>(tw, r * k * step));
        }
        if constexpr (R == 2) dft2<INV>(v);
        else if constexpr (R == 4) dft4<INV>(v);
        else if constexpr (R == 8) dft8<INV>(v);
        else dft_odd<R, INV>(v);
        float2* d = dst + q * ss;
        const int o = jn * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; r++) d[(o + r * Ns) * es] = v[r];
    }
}

// Direct DFT stage for a prime factor R outside the dedicated radices: one work
// item per output (sum over the R twiddled inputs).
template <bool INV>
__device__ __forceinline__ void stage_generic(const float2* src, float2* dst, const FftStage& p, int N,
                                              const FastDiv& fq, int ss, int es, const float2* tw) {
    const int R = p.R, nb = p.nb, Ns = p.Ns, step = p.step;
    const int items = N * (int)fq.d;
    for (int w = threadIdx.x; w < items; w += blockDim.x) {
        const int t = (int)fq.div((unsigned)w), q = w - t * (int)fq.d;  // t: (butterfly j, output m)
        const int j = t % nb, m = t / nb;
        const int k = j % Ns;
        const float2* s = src + q * ss;
        float2 acc = make_float2(0.f, 0.f);
        for (int r = 0; r < R; r++) {
            float2 x = s[(j + r * nb) * es];
            // twiddle w_N^{r k step} and the DFT root w_R^{r m} = w_N^{(r m mod R) nb}
            const int e = (r * k * step + ((r * m) % R) * nb) % N;
            acc = cadd(acc, cmul(x, twid<INV>(tw, e)));
        }
        dst[q * ss + ((j / Ns) * Ns * R + k + m * Ns) * es] = acc;
    }
}

// nseq transforms of length N between buf0 and buf1 (same layout) following the
// host's plan (plan: first stage | count << 24); returns 1 when the result is in
// buf1, 0 when in buf0.  Every thread of the CTA calls it.
template <bool INV>
__device__ int fft_seqs(const Args& a, int plan, float2* buf0, float2* buf1, int N, int nseq, int ss, int es,
                        const float2* tw) {
    const FftStage* st = a.fft_stages + (plan & 0xffffff);
    const int nst = plan >> 24;
    const FastDiv fq(nseq);
    int cur = 0;
    for (int k = 0; k < nst; k++) {
        const FftStage p = st[k];
        const float2* src = cur ? buf1 : buf0;
        float2* dst = cur ? buf0 : buf1;
        if (p.Ns == 1) {
            switch (p.R) {
                case 8: stage_r<8, INV, false>(src, dst, p, fq, ss, es, tw); break;
                case 4: stage_r<4, INV, false>(src, dst, p, fq, ss, es, tw); break;
                case 2: stage_r<2, INV, false>(src, dst, p, fq, ss, es, tw); break;
                case 3: stage_r<3, INV, false>(src, dst, p, fq, ss, es, tw); break;
                case 5: stage_r<5, INV, false>(src, dst, p, fq, ss, es, tw); break;
                case 7: stage_r<7, INV, false>(src, dst, p, fq, ss, es, tw); break;
                default: stage_generic<INV>(src, dst, p, N, fq, ss, es, tw); break;
            }
        } else {
            switch (p.R) {
                case 8: stage_r<8, INV, true>(src, dst, p, fq, ss, es, tw); break;
                case 4: stage_r<4, INV, true>(src, dst, p, fq, ss, es, tw); break;
                case 2: stage_r<2, INV, true>(src, dst, p, fq, ss, es, tw); break;
                case 3: stage_r<3, INV, true>(src, dst, p, fq, ss, es, tw); break;
                case 5: stage_r<5, INV, true>(src, dst, p, fq, ss, es, tw); break;
                case 7: stage_r<7, INV, true>(src, dst, p, fq, ss, es, tw); break;
                default: stage_generic<INV>(src, dst, p, N, fq, ss, es, tw); break;
            }
        }
        __syncthreads();
        cur ^= 1;
    }
    return cur;
}

// Row stride of the z transforms: odd, so that sequence-fastest accesses to
// neighbouring rows fall in different banks.
__device__ __forceinline__ int zrow(int K2) { return K2 | 1; }

// Twiddle tables of the three grid dimensions of a replica, copied to shared memory.
__device__ __forceinline__ void load_tw(const Args& a, const RepDev& R, int d, float2* out) {
    const float2* t = a.fft_tw + R.tw_off[d];
    for (int k = threadIdx.x; k < R.K[d]; k += blockDim.x) cp_async8(out + k, t + k);
}

// Shared memory of the plane kernels: two buffers of a plane of the larger of
// ceil(K1/2) x K2 and K1 x (K2/2 + 1) complex values, and the y and z twiddles.
// The spectrum of a grid is laid out [ky][x][kz] (kz < K2/2 + 1), so that the x
// transforms of one ky read one contiguous slab.
__global__ void __launch_bounds__(kFftThreads, 5) k_fft_zy(Args a) {
    extern __shared__ float2 sh[];
    const int2 pc = a.fft_plane[blockIdx.x];  // (replica, grid * K0 + x)
    const RepDev& R = a.reps[pc.x];
    const int K0 = R.K[0], K1 = R.K[1], K2 = R.K[2], K2h = K2 / 2 + 1, P = (K1 + 1) / 2;
    const int g = pc.y / K0, ix = pc.y - g * K0;
    const int zs = zrow(K2);
    const int plane = (max(P * zs, K1 * K2h) + 1) & ~1;  // even: b1 starts on 16 bytes
    float2* b0 = sh;
    float2* b1 = sh + plane;
    float2* tw1 = sh + 2 * plane;
    float2* tw2 = tw1 + K1;
    load_tw(a, R, 1, tw1);
    load_tw(a, R, 2, tw2);
    const float* G = a.qreal + R.real_off + (size_t)g * K0 * K1 * K2 + (size_t)ix * K1 * K2;
    // the real plane as it lies in memory, into b1 (K1 K2 floats <= 2 P zs)
    float* raw = reinterpret_cast<float*>(b1);
    if ((K2 & 3) == 0 && ((reinterpret_cast<size_t>(G) | reinterpret_cast<size_t>(raw)) & 15) == 0) {
        const int n4 = (K1 * K2) >> 2;
        for (int w = threadIdx.x; w < n4; w += blockDim.x) cp_async16(raw + 4 * w, G + 4 * w);
    } else {
        for (int w = threadIdx.x; w < K1 * K2; w += blockDim.x) cp_async4(raw + w, G + w);
    }
    cp_async_wait_all();
    __syncthreads();
    // rows 2p and 2p + 1 as the real and imaginary parts of row p (charge grids
    // spread by owner hold int32 fixed point)
    const FastDiv fz(K2);
    const bool fixed = a.spread_owner != 0;
    for (int w = threadIdx.x; w < P * K2; w += blockDim.x) {
        const int p = (int)fz.div((unsigned)w), z = w - p * K2;
        float re = raw[(2 * p) * K2 + z];
        float im = 2 * p + 1 < K1 ? raw[(2 * p + 1) * K2 + z] : 0.f;
        if (fixed) {
            re = (float)__float_as_int(re) * (1.0f / kGridScale);
            im = (float)__float_as_int(im) * (1.0f / kGridScale);
        }
        b0[p * zs + z] = make_float2(re, im);
    }
    __syncthreads();
    const int cz = fft_seqs<false>(a, R.fft_plan[2], b0, b1, K2, P, zs, 1, tw2);
    const float2* Z = cz ? b1 : b0;
    float2* S = cz ? b0 : b1;
    // Z = A + iB of two real rows: A_k = (Z_k + conj Z_-k) / 2, B_k = (Z_k - conj Z_-k) / (2i)
    const FastDiv fh(K2h);
    for (int w = threadIdx.x; w < K1 * K2h; w += blockDim.x) {
        const int y = (int)fh.div((unsigned)w), kz = w - y * K2h;
        const int p = y >> 1;
        const float2 zp = Z[p * zs + kz], zm = Z[p * zs + (kz == 0 ? 0 : K2 - kz)];
        S[w] = (y & 1) ? make_float2(0.5f * (zp.y + zm.y), 0.5f * (zm.x - zp.x))
                       : make_float2(0.5f * (zp.x + zm.x), 0.5f * (zp.y - zm.y));
    }
    __syncthreads();
    float2* Zw = const_cast<float2*>(Z);
    const int cy = fft_seqs<false>(a, R.fft_plan[1], S, Zw, K1, K2h, 1, K2h, tw1);
    const float2* Y = cy ? Zw : S;
    float2* out = a.qcplx + R.cplx_off + (size_t)g * K0 * K1 * K2h + (size_t)ix * K2h;
#pragma unroll 4
    for (int w = threadIdx.x; w < K1 * K2h; w += blockDim.x) {
        const int y = (int)fh.div((unsigned)w), kz = w - y * K2h;
        out[(size_t)y * K0 * K2h + kz] = Y[w];
    }
}

__global__ void __launch_bounds__(kFftThreads, 5) k_ifft_yz(Args a) {
    extern __shared__ float2 sh[];
    const int2 pc = a.fft_plane[blockIdx.x];
    const RepDev& R = a.reps[pc.x];
    const int K0 = R.K[0], K1 = R.K[1], K2 = R.K[2], K2h = K2 / 2 + 1, P = (K1 + 1) / 2;
    const int g = pc.y / K0, ix = pc.y - g * K0;
    const int zs = zrow(K2);
    const int plane = (max(P * zs, K1 * K2h) + 1) & ~1;  // even: b1 starts on 16 bytes
    float2* b0 = sh;
    float2* b1 = sh + plane;
    float2* tw1 = sh + 2 * plane;
    float2* tw2 = tw1 + K1;
    load_tw(a, R, 1, tw1);
    load_tw(a, R, 2, tw2);
    const float2* in = a.qcplx + R.cplx_off + (size_t)g * K0 * K1 * K2h + (size_t)ix * K2h;
    const FastDiv fh(K2h);
    for (int w = threadIdx.x; w < K1 * K2h; w += blockDim.x) {
        const int y = (int)fh.div((unsigned)w), kz = w - y * K2h;
        cp_async8(b0 + w, in + (size_t)y * K0 * K2h + kz);
    }
    cp_async_wait_all();
    __syncthreads();
    const int cy = fft_seqs<true>(a, R.fft_plan[1], b0, b1, K1, K2h, 1, K2h, tw1);
    const float2* S = cy ? b1 : b0;
    float2* Z = cy ? b0 : b1;
    // two rows' Hermitian half spectra as one complex row Z = A + iB (the
    // imaginary parts of the k = 0 and k = K2/2 terms are dropped, as a real
    // inverse transform does)
    const FastDiv fz(K2);
    for (int w = threadIdx.x; w < P * K2; w += blockDim.x) {
        const int p = (int)fz.div((unsigned)w), z = w - p * K2;
        const bool up = z > K2 / 2;
        const int kz = up ? K2 - z : z;
        const bool edge = kz == 0 || 2 * kz == K2;
        float2 A = S[(2 * p) * K2h + kz];
        float2 B = 2 * p + 1 < K1 ? S[(2 * p + 1) * K2h + kz] : make_float2(0.f, 0.f);
        if (edge) A.y = B.y = 0.f;
        if (up) {
            A.y = -A.y;
            B.y = -B.y;
        }
        Z[p * zs + z] = make_float2(A.x - B.y, A.y + B.x);
    }
    __syncthreads();
    float2* Sw = const_cast<float2*>(S);
    const int cz = fft_seqs<true>(a, R.fft_plan[2], Z, Sw, K2, P, zs, 1, tw2);
    const float2* Zr = cz ? Sw : Z;
    float* G = a.qreal + R.real_off + (size_t)g * K0 * K1 * K2 + (size_t)ix * K1 * K2;
    if ((K2 & 3) == 0) {
        const int q4 = K2 >> 2;
        const FastDiv f4(q4);
        float4* G4 = reinterpret_cast<float4*>(G);
        for (int w = threadIdx.x; w < K1 * q4; w += blockDim.x) {
            const int y = (int)f4.div((unsigned)w), z4 = w - y * q4;
            const float2* zr = Zr + (y >> 1) * zs + 4 * z4;
            const float2 v0 = zr[0], v1 = zr[1], v2 = zr[2], v3 = zr[3];
            G4[w] = (y & 1) ? make_float4(v0.y, v1.y, v2.y, v3.y) : make_float4(v0.x, v1.x, v2.x, v3.x);
        }
    } else {
        for (int w = threadIdx.x; w < K1 * K2; w += blockDim.x) {
            const int y = (int)fz.div((unsigned)w), z = w - y * K2;
            const float2 v = Zr[(y >> 1) * zs + z];
            G[w] = (y & 1) ? v.y : v.x;
        }
    }
}

// x transforms and the convolution of one (replica, ky, [kz0, kz1)) slab of both
// grids.  Shared layout: M[x][c], c < 2 nz (grid 0's columns, then grid 1's).
__global__ void __launch_bounds__(kFftThreads, 4) k_fft_x_conv(Args a) {
    extern __shared__ float2 sh[];
    __shared__ double red[2][kFftThreads / 32];
    const int4 cc = a.fft_conv[blockIdx.x];  // (replica, ky, kz0, kz1)
    const RepDev& R = a.reps[cc.x];
    const int K0 = R.K[0], K1 = R.K[1], K2 = R.K[2], K2h = K2 / 2 + 1;
    const int ky = cc.y, kz0 = cc.z, nz = cc.w - cc.z, W = 2 * nz;
    float2* b0 = sh;
    float2* b1 = sh + K0 * W;
    float2* tw0 = sh + 2 * K0 * W;
    float* gsh = reinterpret_cast<float*>(tw0 + K0);  // the influence function of the slab, [x][c]
    load_tw(a, R, 0, tw0);
    const size_t C3 = (size_t)K0 * K1 * K2h;
    float2* slab = a.qcplx + R.cplx_off + (size_t)ky * K0 * K2h + kz0;  // [x][kz] of this ky
    // the influence function of this slab (k_influence), in the slab's layout
    const float* Gs = a.influence + R.cplx_off / 2 + (size_t)ky * K0 * K2h + kz0;
    const FastDiv fw(W), fn(nz);
    for (int w = threadIdx.x; w < K0 * W; w += blockDim.x) {
        const int x = (int)fw.div((unsigned)w), c = w - x * W;
        const int g = c >= nz, kz = c - g * nz;
        cp_async8(b0 + w, slab + g * C3 + (size_t)x * K2h + kz);
    }
    for (int w = threadIdx.x; w < K0 * nz; w += blockDim.x) {
        const int x = (int)fn.div((unsigned)w), c = w - x * nz;
        cp_async4(gsh + w, Gs + (size_t)x * K2h + c);
    }
    cp_async_wait_all();
    __syncthreads();
    int cur = fft_seqs<false>(a, R.fft_plan[0], b0, b1, K0, W, 1, W, tw0);
    float2* M = cur ? b1 : b0;
    // influence function G(m) = exp(-pi^2 m^2 / alpha^2) / (pi V m^2 B(m)), B the
    // B-spline moduli; the half spectrum counts kz in (0, K2/2) twice.  Each
    // thread's terms are summed exactly to about 2^-48 (TwoSum), then in FP64.
    float sa = 0.f, ca = 0.f, sb = 0.f, cb = 0.f;
#pragma unroll 2
    for (int w = threadIdx.x; w < K0 * nz; w += blockDim.x) {
        const int x = (int)fn.div((unsigned)w), c = w - x * nz, kz = kz0 + c;
        const float G = gsh[w];
        const float wgt = (kz == 0 || 2 * kz == K2) ? 1.0f : 2.0f;
        const float2 qa = M[x * W + c], qb = M[x * W + nz + c];
        two_sum_add(sa, ca, 0.5f * wgt * G * (qa.x * qa.x + qa.y * qa.y));
        two_sum_add(sb, cb, wgt * G * (qa.x * qb.x + qa.y * qb.y + 0.5f * (qb.x * qb.x + qb.y * qb.y)));
        M[x * W + c] = cscale(qa, G);
        M[x * W + nz + c] = a.full ? cscale(cadd(qa, qb), G) : cscale(qb, G);
    }
    double ea = (double)sa + (double)ca, eb = (double)sb + (double)cb;
    // fixed-order FP64 sums of the energies: warps, then the CTA
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ea += __shfl_xor_sync(0xffffffffu, ea, o);
        eb += __shfl_xor_sync(0xffffffffu, eb, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = ea;
        red[1][threadIdx.x >> 5] = eb;
    }
    __syncthreads();
    if (threadIdx.x < 2) {
        double t = 0.0;
        for (int w = 0; w < kFftThreads / 32; w++) t += red[threadIdx.x][w];
        a.e_part_conv[2 * blockIdx.x + threadIdx.x] = t;
    }
    float2* other = cur ? b0 : b1;
    cur = fft_seqs<true>(a, R.fft_plan[0], M, other, K0, W, 1, W, tw0);
    const float2* out = cur ? other : M;
#pragma unroll 4
    for (int w = threadIdx.x; w < K0 * W; w += blockDim.x) {
        const int x = (int)fw.div((unsigned)w), c = w - x * W;
        const int g = c >= nz, kz = c - g * nz;
        slab[g * C3 + (size_t)x * K2h + kz] = out[w];
    }
}

// Influence function of one replica's grid, in FP64 rounded to FP32, laid out as
// its spectrum ([ky][x][kz], kz < K2/2 + 1): G(m) = exp(-pi^2 m^2 / alpha^2) /
// (pi V m^2 B1(m1) B2(m2) B3(m3)), 0 at m = 0, B the B-spline moduli (Essmann et
// al. 1995).  It depends only on the box, the grid and alpha, so it is computed
// when buffers are made or a box changes, not at every evaluation.
__global__ void k_influence(float* G, const float* mx, const float* my, const float* mz, int K0, int K1, int K2,
                            double r00, double r10, double r11, double r20, double r21, double r22, double vol,
                            double alpha) {
    const int K2h = K2 / 2 + 1;
    const long long n = (long long)K0 * K1 * K2h;
    const double pi = 3.14159265358979323846;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int kz = (int)(e % K2h);
        const long long r = e / K2h;
        const int x = (int)(r % K0), ky = (int)(r / K0);
        const int mxi = x <= K0 / 2 ? x : x - K0, myi = ky <= K1 / 2 ? ky : ky - K1;
        // m = mx a* + my b* + mz c*, the reciprocal vectors being the columns of r
        const double kx = mxi * r00, kyv = mxi * r10 + myi * r11, kzv = mxi * r20 + myi * r21 + kz * r22;
        const double m2 = kx * kx + kyv * kyv + kzv * kzv;
        double g = 0.0;
        if (e != 0 || m2 > 0.0)
            g = m2 > 0.0 ? exp(-pi * pi * m2 / (alpha * alpha)) /
                               (pi * vol * m2 * (double)mx[x] * (double)my[ky] * (double)mz[kz])
                         : 0.0;
        G[e] = (float)g;
    }
}

void launch_influence(float* G, const float* moduli, const int* mod_off, const int* K, const double* recip,
                      double volume, double alpha, cudaStream_t s) {
    const long long n = (long long)K[0] * K[1] * (K[2] / 2 + 1);
    const int blocks = (int)std::min<long long>((n + 255) / 256, 4096);
    k_influence<<<blocks, 256, 0, s>>>(G, moduli + mod_off[0], moduli + mod_off[1], moduli + mod_off[2], K[0], K[1],
                                      K[2], recip[0], recip[1], recip[2], recip[3], recip[4], recip[5], volume, alpha);
}

int fft_plane_smem_bytes(int K1, int K2) {
    const int P = (K1 + 1) / 2, K2h = K2 / 2 + 1, zs = K2 | 1;
    const int plane = ((P * zs > K1 * K2h ? P * zs : K1 * K2h) + 1) & ~1;
    return (int)sizeof(float2) * (2 * plane + K1 + K2);
}

// Radices 8 (as many as divide N), then 4 or 2 for the rest of the power of two,
// then 3, 5, 7 and any other prime factor, smallest first.
int fft_plan_stages(int N, std::vector<FftStage>& out) {
    std::vector<int> rad;
    int n = N;
    while (n % 8 == 0) { rad.push_back(8); n /= 8; }
    if (n % 4 == 0) { rad.push_back(4); n /= 4; }
    if (n % 2 == 0) { rad.push_back(2); n /= 2; }
    for (int p = 3; n > 1; p += 2)
        while (n % p == 0) { rad.push_back(p); n /= p; }
    const int first = (int)out.size();
    int Ns = 1;
    for (int R : rad) {
        FftStage st{};
        st.R = R;
        st.Ns = Ns;
        st.nb = N / R;
        st.step = N / (Ns * R);
        st.mNs = Ns > 1 ? (unsigned)((0x100000000ull + (unsigned long long)Ns - 1) / (unsigned long long)Ns) : 0u;
        out.push_back(st);
        Ns *= R;
    }
    return first | (int)rad.size() << 24;
}

int fft_conv_smem_bytes(int K0, int nz) {
    return (int)sizeof(float2) * (2 * K0 * 2 * nz + K0) + (int)sizeof(float) * ((K0 * nz + 1) & ~1);
}

void launch_fft_forward(const Args& a, cudaStream_t s) {
    if (a.fft_plane_ctas <= 0) return;
    cudaFuncSetAttribute(k_fft_zy, cudaFuncAttributeMaxDynamicSharedMemorySize, a.fft_plane_smem);
    k_fft_zy<<<a.fft_plane_ctas, kFftThreads, a.fft_plane_smem, s>>>(a);
}

void launch_fft_conv(const Args& a, cudaStream_t s) {
    if (a.conv_ctas <= 0) return;
    cudaFuncSetAttribute(k_fft_x_conv, cudaFuncAttributeMaxDynamicSharedMemorySize, a.fft_conv_smem);
    k_fft_x_conv<<<a.conv_ctas, kFftThreads, a.fft_conv_smem, s>>>(a);
}

void launch_fft_inverse(const Args& a, cudaStream_t s) {
    if (a.fft_plane_ctas <= 0) return;
    cudaFuncSetAttribute(k_ifft_yz, cudaFuncAttributeMaxDynamicSharedMemorySize, a.fft_plane_smem);
    k_ifft_yz<<<a.fft_plane_ctas, kFftThreads, a.fft_plane_smem, s>>>(a);
}

}  // namespace atm
