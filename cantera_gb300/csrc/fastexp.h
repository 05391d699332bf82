// fastexp.h - FP64 exponential with the polynomial on the integer pipe.
//
// On GB300 the FP64 unit issues one warp instruction per 64 cycles per SM sub-partition,
// while 32-bit integer multiply-adds run at FP32-like rates.  This exponential keeps only
// the argument reduction in FP64 (four operations) and evaluates everything else in Q63
// fixed point with 64x64->128-bit integer products:
//
//   x = (64 e + j) ln2/64 + r,  |r| <= ln2/128          (Tang, ACM TOMS 15(2) 1989)
//   exp(x) = 2^e * 2^(j/64) * (1 + p(r)),  p(r) = r + r^2/2 + r^3/6 + r^4/24 + r^5/120
//
// The Taylor truncation error is below 4e-17, the fixed-point roundings below 1e-18, the
// table 2^(j/64) is correctly rounded to 64 bits; the result is rounded once to double
// (round half up), so it stays within one unit in the last place of exp(x).
//
// A value is carried as XVal {u, e} = u / 2^63 * 2^e with u in [2^63, 2^64): products of
// such values (the equilibrium constants multiply several species exponentials) stay on
// the integer pipe and are converted to double once.
//
// Works on the host too (128-bit products through unsigned __int128), for tests.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define GBX_HD __host__ __device__ __forceinline__
#else
#define GBX_HD inline
#endif

namespace gbchem {

struct XVal {
    uint64_t u;   // mantissa in [2^63, 2^64); 0 for the value 0
    int e;        // binary exponent
};

GBX_HD uint64_t gbx_umulhi(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * (unsigned __int128)b) >> 64);
#endif
}
GBX_HD int64_t gbx_mulhi(int64_t a, int64_t b) {
#ifdef __CUDA_ARCH__
    return __mul64hi(a, b);
#else
    return (int64_t)(((__int128)a * (__int128)b) >> 64);
#endif
}
// (a * b) >> 63 for signed Q63 operands (floor)
GBX_HD int64_t gbx_mulq63(int64_t a, int64_t b) {
    const uint64_t hi = (uint64_t)gbx_mulhi(a, b);
    const uint64_t lo = (uint64_t)a * (uint64_t)b;
    return (int64_t)((hi << 1) | (lo >> 63));
}
GBX_HD int64_t gbx_bits(double x) {
#ifdef __CUDA_ARCH__
    return __double_as_longlong(x);
#else
    int64_t b;
    memcpy(&b, &x, 8);
    return b;
#endif
}
GBX_HD double gbx_double(int64_t b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double(b);
#else
    double x;
    memcpy(&x, &b, 8);
    return x;
#endif
}

// 2^(j/64) * 2^63, correctly rounded.  Device code reads a copy in shared memory (lanes
// index it at random; constant memory would serialise them), see gbx_load_table.
#ifdef __CUDACC__
__device__ __constant__
#else
static const
#endif
uint64_t gbx_t63[64] = {
    0x8000000000000000ULL, 0x8164d1f3bc030773ULL, 0x82cd8698ac2ba1d7ULL, 0x843a28c3acde4046ULL,
    0x85aac367cc487b15ULL, 0x871f61969e8d1010ULL, 0x88980e8092da8527ULL, 0x8a14d575496efd9aULL,
    0x8b95c1e3ea8bd6e7ULL, 0x8d1adf5b7e5ba9e6ULL, 0x8ea4398b45cd53c0ULL, 0x9031dc431466b1dcULL,
    0x91c3d373ab11c336ULL, 0x935a2b2f13e6e92cULL, 0x94f4efa8fef70961ULL, 0x96942d3720185a00ULL,
    0x9837f0518db8a96fULL, 0x99e0459320b7fa65ULL, 0x9b8d39b9d54e5539ULL, 0x9d3ed9a72cffb751ULL,
    0x9ef5326091a111aeULL, 0xa0b0510fb9714fc2ULL, 0xa27043030c496819ULL, 0xa43515ae09e6809eULL,
    0xa5fed6a9b15138eaULL, 0xa7cd93b4e965356aULL, 0xa9a15ab4ea7c0ef8ULL, 0xab7a39b5a93ed337ULL,
    0xad583eea42a14ac6ULL, 0xaf3b78ad690a4375ULL, 0xb123f581d2ac2590ULL, 0xb311c412a9112489ULL,
    0xb504f333f9de6484ULL, 0xb6fd91e328d17791ULL, 0xb8fbaf4762fb9ee9ULL, 0xbaff5ab2133e45fbULL,
    0xbd08a39f580c36bfULL, 0xbf1799b67a731083ULL, 0xc12c4cca66709456ULL, 0xc346ccda24976407ULL,
    0xc5672a115506daddULL, 0xc78d74c8abb9b15dULL, 0xc9b9bd866e2f27a3ULL, 0xcbec14fef2727c5dULL,
    0xce248c151f8480e4ULL, 0xd06333daef2b2595ULL, 0xd2a81d91f12ae45aULL, 0xd4f35aabcfedfa1fULL,
    0xd744fccad69d6af4ULL, 0xd99d15c278afd7b6ULL, 0xdbfbb797daf23755ULL, 0xde60f4825e0e9124ULL,
    0xe0ccdeec2a94e111ULL, 0xe33f8972be8a5a51ULL, 0xe5b906e77c8348a8ULL, 0xe8396a503c4bdc68ULL,
    0xeac0c6e7dd24392fULL, 0xed4f301ed9942b84ULL, 0xefe4b99bdcdaf5cbULL, 0xf281773c59ffb13aULL,
    0xf5257d152486cc2cULL, 0xf7d0df730ad13bb9ULL, 0xfa83b2db722a033aULL, 0xfd3e0c0cf486c175ULL};

#ifdef __CUDACC__
// copy the table into a block's shared array (all threads call; includes a barrier)
__device__ __forceinline__ void gbx_load_table(uint64_t* tab) {
    for (int j = threadIdx.x; j < 64; j += blockDim.x) tab[j] = gbx_t63[j];
    __syncthreads();
}
#endif

// |x| >= 700, infinity or NaN: such arguments take the library exp
GBX_HD bool gbx_big(double x) {
    return (int)(((uint64_t)gbx_bits(x) >> 32) & 0x7fffffffu) >= 0x4085E000;
}

// FP64 argument reduction: x = k ln2/64 + r (k integer, |r| <= ln2/128 + tiny)
GBX_HD double gbx_reduce(double x, int& k) {
    const double shifter = 6755399441055744.0;            // 1.5 * 2^52
    const double t = fma(x, 92.33248261689366, shifter);   // x * 64/ln2, rounded to an integer
    k = (int)(uint32_t)((uint64_t)gbx_bits(t) & 0xffffffffu);
    const double kd = t - shifter;
    double r = fma(-kd, 0.010830424726009369, x);          // ln2/64, leading 24 bits
    return fma(-kd, -2.9760223436840126e-11, r);           // ln2/64, next bits
}

// |r| < 2^-7 as a signed Q63 integer
GBX_HD int64_t gbx_q63(double r) {
    const int64_t b = gbx_bits(r);
    const int E = (int)((b >> 52) & 0x7ff);
    if (E == 0) return 0;
    const uint64_t m = ((uint64_t)b & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);   // r = m 2^(E-1075)
    const int sh = E - 1012;                                               // Q63: m 2^(E-1012)
    uint64_t q = sh >= 0 ? (m << sh) : (sh > -64 ? (m >> -sh) : 0ULL);
    return b < 0 ? -(int64_t)q : (int64_t)q;
}

// exp(r) - 1 in Q63 for |r| < 2^-7 given in Q63
GBX_HD int64_t gbx_expm1_q63(int64_t r) {
    int64_t s = 0x0555555555555555LL + gbx_mulq63(r, 0x0111111111111111LL);   // 1/24 + r/120
    s = 0x1555555555555555LL + gbx_mulq63(r, s);                               // 1/6 + ...
    s = 0x4000000000000000LL + gbx_mulq63(r, s);                               // 1/2 + ...
    const int64_t q = gbx_mulq63(r, s);                                        // r/2 + ...
    return r + gbx_mulq63(r, q);
}

// 2^(j/64) (1 + p) 2^e with k = 64 e + j
GBX_HD XVal gbx_assemble(int k, int64_t p, const uint64_t* tab) {
    const uint64_t onep = 0x8000000000000000ULL + (uint64_t)p;   // (1 + p) in Q63
    const uint64_t hi = gbx_umulhi(tab[k & 63], onep);           // value * 2^62, in [0.99, 1.99)
    XVal v;
    if (hi >> 62) { v.u = hi << 1; v.e = k >> 6; }
    else { v.u = hi << 2; v.e = (k >> 6) - 1; }
    return v;
}

// exp(x) and exp(-x) as XVal; requires !gbx_big(x)
GBX_HD void gbx_exp_pm(double x, XVal& ep, XVal& em, const uint64_t* tab) {
    int k;
    const double r = gbx_reduce(x, k);
    const int64_t rq = gbx_q63(r);
    ep = gbx_assemble(k, gbx_expm1_q63(rq), tab);
    em = gbx_assemble(-k, gbx_expm1_q63(-rq), tab);
}

// product of two XVal
GBX_HD XVal gbx_mul(XVal a, XVal b) {
    const uint64_t hi = gbx_umulhi(a.u, b.u);   // value * 2^62 in [1, 4)
    XVal v;
    if (hi >> 63) { v.u = hi; v.e = a.e + b.e + 1; }
    else { v.u = hi << 1; v.e = a.e + b.e; }
    return v;
}

// u / 2^63 rounded to double, in [1, 2] (the exponent is applied separately)
GBX_HD double gbx_mant(uint64_t u, int& carry) {
    carry = 0;
    if (u >= 0xFFFFFFFFFFFFFC00ULL) { carry = 1; return 1.0; }
    uint64_t m = (u + 0x400ULL) >> 11;                    // 53 bits, round half up
    if (m >> 53) { carry = 1; return 1.0; }
    return gbx_double((int64_t)((1023ULL << 52) | (m & 0xFFFFFFFFFFFFFULL)));
}

// XVal to double; the caller guarantees a normal result (|e| < 1000)
GBX_HD double gbx_todouble(XVal v) {
    int c;
    const double m = gbx_mant(v.u, c);
    return gbx_double(gbx_bits(m) + ((int64_t)(v.e + c) << 52));
}

// exp(x) in double
GBX_HD double gbx_exp(double x, const uint64_t* tab) {
    if (gbx_big(x)) return exp(x);
    int k;
    const double r = gbx_reduce(x, k);
    return gbx_todouble(gbx_assemble(k, gbx_expm1_q63(gbx_q63(r)), tab));
}

}  // namespace gbchem
