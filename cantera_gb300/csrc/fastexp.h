// fastexp.h - FP64 exponential and logarithm with the polynomials on the integer pipe.
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
// The logarithm (gbx_log) works the same way: the exponent and a 128-entry table split x,
// the remainder's series runs in Q63, the sum is formed in 128-bit Q64 fixed point and
// rounded to double once (no FP64 instruction at all).  Its error is below 2^-60 absolute
// (within about one unit in the last place wherever |ln x| > 1/256): it serves the
// engine's uses, whose results enter exponentials and sums, not as a general log near 1.
//
// Works on the host too (128-bit products through unsigned __int128), for tests.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

// Non-inline functions of these headers have internal linkage in the kernel modules that
// compile the same code again (kernels_x.cu, krylov.cu, krylov32.cu): their host-side stubs must not
// collide at link time.
#if defined(GB_KERNELS_EXTRA) || defined(GB_KERNELS_KRYLOV)
#define GB_TU_LOCAL static
#else
#define GB_TU_LOCAL
#endif
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

// Logarithm tables, generated from their definitions in 80-digit decimal arithmetic:
// gbx_linv[j] = ceil(2^64 / (128 + j)), gbx_lnf[j] = round(ln(1 + j/128) * 2^64).
#ifdef __CUDACC__
__device__ __constant__
#else
static const
#endif
uint64_t gbx_linv[128] = {
    0x0200000000000000ULL, 0x01fc07f01fc07f02ULL, 0x01f81f81f81f81f9ULL, 0x01f44659e4a42716ULL,
    0x01f07c1f07c1f07dULL, 0x01ecc07b301ecc08ULL, 0x01e9131abf0b7673ULL, 0x01e573ac901e573bULL,
    0x01e1e1e1e1e1e1e2ULL, 0x01de5d6e3f8868a5ULL, 0x01dae6076b981dafULL, 0x01d77b654b82c33aULL,
    0x01d41d41d41d41d5ULL, 0x01d0cb58f6ec0744ULL, 0x01cd85689039b0aeULL, 0x01ca4b3055ee1911ULL,
    0x01c71c71c71c71c8ULL, 0x01c3f8f01c3f8f02ULL, 0x01c0e070381c0e08ULL, 0x01bdd2b899406f75ULL,
    0x01bacf914c1bacfaULL, 0x01b7d6c3dda338b3ULL, 0x01b4e81b4e81b4e9ULL, 0x01b2036406c80d91ULL,
    0x01af286bca1af287ULL, 0x01ac5701ac5701adULL, 0x01a98ef606a63bd9ULL, 0x01a6d01a6d01a6d1ULL,
    0x01a41a41a41a41a5ULL, 0x01a16d3f97a4b01bULL, 0x019ec8e951033d92ULL, 0x019c2d14ee4a101aULL,
    0x019999999999999aULL, 0x01970e4f80cb8728ULL, 0x01948b0fcd6e9e07ULL, 0x01920fb49d0e228eULL,
    0x018f9c18f9c18f9dULL, 0x018d3018d3018d31ULL, 0x018acb90f6bf3a9bULL, 0x01886e5f0abb049aULL,
    0x0186186186186187ULL, 0x0183c977ab2bedd3ULL, 0x0181818181818182ULL, 0x017f405fd017f406ULL,
    0x017d05f417d05f42ULL, 0x017ad2208e0ecc36ULL, 0x0178a4c8178a4c82ULL, 0x01767dce434a9b11ULL,
    0x01745d1745d1745eULL, 0x01724287f46debc1ULL, 0x01702e05c0b81703ULL, 0x016e1f76b4337c6dULL,
    0x016c16c16c16c16dULL, 0x016a13cd15372905ULL, 0x0168168168168169ULL, 0x01661ec6a5122f91ULL,
    0x01642c8590b21643ULL, 0x01623fa7701623fbULL, 0x0160581605816059ULL, 0x015e75bb8d015e76ULL,
    0x015c9882b9310573ULL, 0x015ac056b015ac06ULL, 0x0158ed2308158ed3ULL, 0x01571ed3c506b39bULL,
    0x0155555555555556ULL, 0x015390948f40feadULL, 0x0151d07eae2f8152ULL, 0x0150150150150151ULL,
    0x014e5e0a72f05398ULL, 0x014cab88725af6e8ULL, 0x014afd6a052bf5a9ULL, 0x0149539e3b2d066fULL,
    0x0147ae147ae147afULL, 0x01460cbc7f5cf9a2ULL, 0x01446f86562d9fafULL, 0x0142d6625d51f86fULL,
    0x0141414141414142ULL, 0x013fb013fb013fb1ULL, 0x013e22cbce4a9028ULL, 0x013c995a47babe75ULL,
    0x013b13b13b13b13cULL, 0x013991c2c187f634ULL, 0x0138138138138139ULL, 0x013698df3de0747aULL,
    0x013521cfb2b78c14ULL, 0x0133ae45b57bcb1fULL, 0x01323e34a2b10bf7ULL, 0x0130d190130d1902ULL,
    0x012f684bda12f685ULL, 0x012e025c04b80971ULL, 0x012c9fb4d812c9fcULL, 0x012b404ad012b405ULL,
    0x0129e4129e4129e5ULL, 0x01288b01288b0129ULL, 0x0127350b88127351ULL, 0x0125e22708092f12ULL,
    0x0124924924924925ULL, 0x0123456789abcdf1ULL, 0x0121fb78121fb782ULL, 0x0120b470c67c0d89ULL,
    0x011f7047dc11f705ULL, 0x011e2ef3b3fb8745ULL, 0x011cf06ada2811d0ULL, 0x011bb4a4046ed291ULL,
    0x011a7b9611a7b962ULL, 0x0119453808ca29c1ULL, 0x0118118118118119ULL, 0x0116e0689427378fULL,
    0x0115b1e5f75270d1ULL, 0x011485f0e0acd3b7ULL, 0x01135c81135c8114ULL, 0x0112358e75d30337ULL,
    0x0111111111111112ULL, 0x010fef010fef0110ULL, 0x010ecf56be69c8feULL, 0x010db20a88f4695aULL,
    0x010c9714fbcda3adULL, 0x010b7e6ec259dc7aULL, 0x010a6810a6810a69ULL, 0x010953f390109540ULL,
    0x0108421084210843ULL, 0x01073260a47f7c67ULL, 0x010624dd2f1a9fbfULL, 0x0105197f7d734042ULL,
    0x0104104104104105ULL, 0x0103091b51f5e1a5ULL, 0x0102040810204082ULL, 0x0101010101010102ULL,
};
#ifdef __CUDACC__
__device__ __constant__
#else
static const
#endif
uint64_t gbx_lnf[128] = {
    0x0000000000000000ULL, 0x01fe02a6b1067890ULL, 0x03f815161f807c7aULL, 0x05ee46c1f56c46aaULL,
    0x07e0a6c39e0cc013ULL, 0x09cf43dcff5eafd5ULL, 0x0bba2c7b196e7e23ULL, 0x0da16eb88cb8df61ULL,
    0x0f85186008b15331ULL, 0x116536eea37ae0e8ULL, 0x1341d7961bd1d093ULL, 0x151b073f06183f69ULL,
    0x16f0d28ae56b4b9cULL, 0x18c345d6319b20f6ULL, 0x1a926d3a4ad56365ULL, 0x1c5e548f5bc74316ULL,
    0x1e27076e2af2e5eaULL, 0x1fec9131dbeabaaaULL, 0x21aefcf9a11cb2cdULL, 0x236e55aa5ecf4052ULL,
    0x252aa5f03fea4698ULL, 0x26e3f8403d1ee878ULL, 0x289a56d996fa3cd0ULL, 0x2a4dcbc743686f46ULL,
    0x2bfe60e14f27a791ULL, 0x2dac1fce33a4391bULL, 0x2f57120421b21238ULL, 0x30ff40ca41922120ULL,
    0x32a4b539e8ad68edULL, 0x3447783fc56ac632ULL, 0x35e7929d017fe5b2ULL, 0x37850ce85b19ac54ULL,
    0x391fef8f35344358ULL, 0x3ab842d69f7722b7ULL, 0x3c4e0edc55e5cbd4ULL, 0x3de15b97b8b26ca4ULL,
    0x3f7230dabc7c551bULL, 0x41009652d341036cULL, 0x428c9389ce438d7eULL, 0x44162fe6b92b5462ULL,
    0x459d72aeae98380eULL, 0x47226305a667ebefULL, 0x48a507ef3de59689ULL, 0x4a25684f7a1a8d7bULL,
    0x4ba38aeb8474c271ULL, 0x4d1f766a61f55359ULL, 0x4e993155a517a71dULL, 0x5010c21a1a9f8ef4ULL,
    0x51862f08717b09f4ULL, 0x52f97e55dde2836dULL, 0x546ab61cb7e0b427ULL, 0x55d9dc5d1569b152ULL,
    0x5746f6fd60272942ULL, 0x58b20bcae71e54beULL, 0x5a1b207a6c52bb11ULL, 0x5b823aa8ae878e30ULL,
    0x5ce75fdaef401a74ULL, 0x5e4a957f751e89f0ULL, 0x5fabe0ee0abf0d93ULL, 0x610b47687a2c5d25ULL,
    0x6268ce1b05096ad7ULL, 0x63c47a1cd98b1df8ULL, 0x651e5070845beae9ULL, 0x667656045f822b2fULL,
    0x67cc8fb2fe612fcbULL, 0x6921024396ec28b0ULL, 0x6a73b26a68212635ULL, 0x6bc4a4c91de1ac45ULL,
    0x6d13ddef323d8a33ULL, 0x6e61625a4c43ed66ULL, 0x6fad36769c6defdeULL, 0x70f75e9f36b535cfULL,
    0x723fdf1e6a6886b1ULL, 0x7386bc2e17cfadeeULL, 0x74cbf9f803af5587ULL, 0x760f9c9628bcf941ULL,
    0x7751a813071282fcULL, 0x78922069f1b09873ULL, 0x79d109875a1e1f8eULL, 0x7b0e67491a33005dULL,
    0x7c4a3d7ebc1bb2cdULL, 0x7d848fe9c0a2b185ULL, 0x7ebd623de3cc7b67ULL, 0x7ff4b8215fd26156ULL,
    0x812a952d2e87f635ULL, 0x825efced49369330ULL, 0x8391f2e0e6fa0273ULL, 0x84c37a7ab9a905c9ULL,
    0x85f39721295415b5ULL, 0x87224c2e8e645fb7ULL, 0x884f9cf16a64b7efULL, 0x897b8cac9f7de298ULL,
    0x8aa61e97a6af4d4cULL, 0x8bcf55dec4cd05feULL, 0x8cf735a33e4b7663ULL, 0x8e1dc0fb89e125e5ULL,
    0x8f42faf3820681efULL, 0x9066e68c955b6c9bULL, 0x918986bdf5fa1417ULL, 0x92aade74c7be59e0ULL,
    0x93caf0944d88d75cULL, 0x94e9bff615845643ULL, 0x96074f6a24745dccULL, 0x9723a1b720134203ULL,
    0x983eb99a7885f0feULL, 0x995899c890eb8990ULL, 0x9a7144ece70e98b7ULL, 0x9b88bdaa3a3dae2fULL,
    0x9c9f069ab150cd4eULL, 0x9db4224fffe1157cULL, 0x9ec813538ab7d520ULL, 0x9fdadc268b7a12daULL,
    0xa0ec7f4233957323ULL, 0xa1fcff17ce733bd4ULL, 0xa30c5e10e2f613e8ULL, 0xa41a9e8f5446fb9fULL,
    0xa527c2ed81f5d811ULL, 0xa633cd7e6771cd8bULL, 0xa73ec08dbadd84e6ULL, 0xa8489e600b435a5eULL,
    0xa9516932de2d5774ULL, 0xaa59233ccca4bd49ULL, 0xab5fcead9f9cca09ULL, 0xac656dae6bcc4985ULL,
    0xad6a0261acf967d9ULL, 0xae6d8ee360bb2468ULL, 0xaf70154920b3ab87ULL, 0xb07197a23c46c654ULL,
};
constexpr uint64_t kGbxLn2Hi = 0xb17217f7d1cf79abULL;   // floor(ln2 * 2^64)
constexpr uint64_t kGbxLn2Lo = 0xc9e3b39803f2f6afULL;   // the next 64 bits of ln2
// layout of the combined table: exp [0, 64), 1/(128+j) [64, 192), ln(1+j/128) [192, 320)
constexpr int kGbxLogInv = 64, kGbxLogTab = 192, kGbxTableWords = 320;

#ifdef __CUDACC__
// copy the tables into a block's shared array of kGbxTableWords (all threads call;
// includes a barrier)
__device__ __forceinline__ void gbx_load_table(uint64_t* tab) {
    for (int j = threadIdx.x; j < kGbxTableWords; j += blockDim.x)
        tab[j] = j < 64 ? gbx_t63[j] : (j < kGbxLogTab ? gbx_linv[j - kGbxLogInv] : gbx_lnf[j - kGbxLogTab]);
    __syncthreads();
}
#endif
#ifndef __CUDACC__
// the same layout on the host (tests)
inline void gbx_host_table(uint64_t* tab) {
    for (int j = 0; j < kGbxTableWords; j++)
        tab[j] = j < 64 ? gbx_t63[j] : (j < kGbxLogTab ? gbx_linv[j - kGbxLogInv] : gbx_lnf[j - kGbxLogTab]);
}
#endif

// |x| >= 700, infinity or NaN: such arguments take the library exp
GBX_HD bool gbx_big(double x) {
    return (int)(((uint64_t)gbx_bits(x) >> 32) & 0x7fffffffu) >= 0x4085E000;
}

// the library functions for the rare arguments, out of line (one copy of their code)
#ifdef __CUDACC__
GB_TU_LOCAL __device__ __noinline__ double gbx_exp_slow(double x) { return exp(x); }
GB_TU_LOCAL __device__ __noinline__ double gbx_log_slow(double x) { return log(x); }
#endif
#ifdef __CUDA_ARCH__
#define GBX_EXP_SLOW(x) gbx_exp_slow(x)
#define GBX_LOG_SLOW(x) gbx_log_slow(x)
#else
#define GBX_EXP_SLOW(x) exp(x)
#define GBX_LOG_SLOW(x) log(x)
#endif
// the exponential and the logarithm are called from many places: one out-of-line copy
// each on the device keeps the kernels' code (and instruction-cache footprint) small
#ifdef __CUDACC__
#define GBX_HD_NOINLINE __host__ __device__ __noinline__
#else
#define GBX_HD_NOINLINE inline
#endif

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
GB_TU_LOCAL GBX_HD_NOINLINE double gbx_exp(double x, const uint64_t* tab) {
    if (gbx_big(x)) return GBX_EXP_SLOW(x);
    int k;
    const double r = gbx_reduce(x, k);
    return gbx_todouble(gbx_assemble(k, gbx_expm1_q63(gbx_q63(r)), tab));
}


// ---- logarithm ----------------------------------------------------------------------

GBX_HD int gbx_clz64(uint64_t v) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}

// signed Q64 fixed-point value (128 bits) to double, rounded half up in magnitude
GBX_HD double gbx_q64_to_double(__int128 v) {
    if (v == 0) return 0.0;
    const bool neg = v < 0;
    const unsigned __int128 a = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
    const uint64_t hi = (uint64_t)(a >> 64), lo = (uint64_t)a;
    const int lz = hi ? gbx_clz64(hi) : 64 + gbx_clz64(lo);
    const uint64_t top = (uint64_t)((a << lz) >> 64);     // leading one at bit 63
    uint64_t m = (top >> 11) + ((top >> 10) & 1ULL);
    int ex = 63 - lz;                                     // value = a * 2^-64
    if (m >> 53) { m >>= 1; ex++; }
    const uint64_t bits = ((uint64_t)(ex + 1023) << 52) | (m & 0xFFFFFFFFFFFFFULL) |
                          (neg ? 0x8000000000000000ULL : 0ULL);
    return gbx_double((int64_t)bits);
}

// ln(x); positive normal x on the integer pipe, anything else through the library log
GB_TU_LOCAL GBX_HD_NOINLINE double gbx_log(double x, const uint64_t* tab) {
    const int64_t b = gbx_bits(x);
    if ((uint64_t)(b - 0x0010000000000000LL) >= 0x7FE0000000000000ULL) return GBX_LOG_SLOW(x);
    const int e = (int)(b >> 52) - 1023;
    const uint64_t mant = (uint64_t)b & 0xFFFFFFFFFFFFFULL;
    const int j = (int)(mant >> 45);
    const uint64_t D = mant & 0x1FFFFFFFFFFFULL;                  // m - (1 + j/128), times 2^52
    const int64_t r = (int64_t)(gbx_umulhi(D << 19, tab[kGbxLogInv + j]) >> 1);   // Q63, < 2^-7
    int64_t t = 0x1000000000000000LL;                             // 1/8
    t = 0x1249249249249249LL - gbx_mulq63(r, t);                  // 1/7 - r t
    t = 0x1555555555555555LL - gbx_mulq63(r, t);                  // 1/6
    t = 0x1999999999999999LL - gbx_mulq63(r, t);                  // 1/5
    t = 0x2000000000000000LL - gbx_mulq63(r, t);                  // 1/4
    t = 0x2AAAAAAAAAAAAAAALL - gbx_mulq63(r, t);                  // 1/3
    t = 0x4000000000000000LL - gbx_mulq63(r, t);                  // 1/2
    const int64_t p = r - gbx_mulq63(r, gbx_mulq63(r, t));        // ln(1 + r), Q63
    __int128 acc = (__int128)e * (__int128)kGbxLn2Hi + (((__int128)e * (__int128)kGbxLn2Lo) >> 64);
    acc += (__int128)tab[kGbxLogTab + j];
    acc += (__int128)p * 2;
    return gbx_q64_to_double(acc);
}

GBX_HD double gbx_log10(double x, const uint64_t* tab) { return gbx_log(x, tab) * 0.4342944819032518; }

}  // namespace gbchem
