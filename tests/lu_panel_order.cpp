// The integrator's dense LU beyond 64 components (kernels.cu) in two orders of the same
// operations: unblocked right-looking (luRight here) and in panels of four (luRightPanel4), with
// explicit fused multiply-adds as the device code has them.  The two must give the same
// factors, pivots and reciprocal diagonals bit for bit on random matrices (sizes 1-128,
// sparse and dense, row interchanges, rank-deficient ones).  Exit status 0: identical.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>
template <typename MT> static uint64_t key(MT x) { double d = x; uint64_t u; memcpy(&u, &d, 8); return u & 0x7FFFFFFFFFFFFFFFULL; }
template <typename MT>
bool luRight(MT* a, int N, int ld, int* piv, double* dinv) {
    for (int i = 0; i < N; i++) piv[i] = i;
    for (int k = 0; k < N; k++) {
        uint64_t bv = 0; int bi = N;
        for (int i = k; i < N; i++) { uint64_t v = key(a[(size_t)i * ld + k]); if (v > bv || bi == N) { bv = v; bi = i; } }
        if (bv == 0) return false;
        if (bi != k) { for (int j = 0; j < N; j++) std::swap(a[(size_t)k * ld + j], a[(size_t)bi * ld + j]); std::swap(piv[k], piv[bi]); }
        MT inv = (MT)1 / a[(size_t)k * ld + k]; dinv[k] = (double)inv;
        for (int i = k + 1; i < N; i++) a[(size_t)i * ld + k] *= inv;
        for (int j = k + 1; j < N; j++) { MT u = a[(size_t)k * ld + j];
            for (int i = k + 1; i < N; i++) a[(size_t)i * ld + j] = std::fma(-a[(size_t)i * ld + k], u, a[(size_t)i * ld + j]); }
    }
    return true;
}
template <typename MT>
bool luPanel(MT* a, int N, int ld, int* piv, double* dinv) {
    const int B = 4;
    for (int i = 0; i < N; i++) piv[i] = i;
    for (int k0 = 0; k0 < N; k0 += B) {
        int kend = std::min(k0 + B, N);
        for (int k = k0; k < kend; k++) {
            uint64_t bv = 0; int bi = N;
            for (int i = k; i < N; i++) { uint64_t v = key(a[(size_t)i * ld + k]); if (v > bv || bi == N) { bv = v; bi = i; } }
            if (bv == 0) return false;
            if (bi != k) { for (int j = 0; j < N; j++) std::swap(a[(size_t)k * ld + j], a[(size_t)bi * ld + j]); std::swap(piv[k], piv[bi]); }
            MT inv = (MT)1 / a[(size_t)k * ld + k]; dinv[k] = (double)inv;
            for (int i = k + 1; i < N; i++) { MT* r = a + (size_t)i * ld; MT l = r[k] * inv; r[k] = l;
                for (int j = k + 1; j < kend; j++) r[j] = std::fma(-l, a[(size_t)k * ld + j], r[j]); }
        }
        int nb = kend - k0;
        for (int j = kend; j < N; j++) {
            MT u[B] = {0, 0, 0, 0};
            for (int p = 0; p < nb; p++) u[p] = a[(size_t)(k0 + p) * ld + j];
            for (int p = 1; p < nb; p++) { const MT* r = a + (size_t)(k0 + p) * ld + k0;
                for (int q = 0; q < p; q++) u[p] = std::fma(-r[q], u[q], u[p]); a[(size_t)(k0 + p) * ld + j] = u[p]; }
            for (int i = kend; i < N; i++) { MT* row = a + (size_t)i * ld; MT v = row[j];
                for (int p = 0; p < nb; p++) v = std::fma(-row[k0 + p], u[p], v); row[j] = v; }
        }
    }
    return true;
}
template <typename MT> int run(std::mt19937_64& g, int trials) {
    int bad = 0;
    std::uniform_int_distribution<int> dn(1, 128);
    std::normal_distribution<double> nd;
    std::uniform_real_distribution<double> ud(0, 1);
    for (int t = 0; t < trials; t++) {
        int N = dn(g), ld = N + (t % 3);
        std::vector<MT> A((size_t)N * ld), B2;
        double dens = ud(g);
        for (int i = 0; i < N; i++) for (int j = 0; j < N; j++) {
            double v = (ud(g) < dens) ? nd(g) * std::pow(10.0, 6 * ud(g) - 3) : 0.0;
            if (i == j && ud(g) < 0.7) v += 1.0;
            A[(size_t)i * ld + j] = (MT)v; }
        if (t % 7 == 0 && N > 2) for (int j = 0; j < N; j++) A[(size_t)1 * ld + j] = A[(size_t)0 * ld + j] * (MT)2;  // rank deficiency
        B2 = A;
        std::vector<int> p1(N), p2(N); std::vector<double> d1(N), d2(N);
        bool o1 = luRight(A.data(), N, ld, p1.data(), d1.data()), o2 = luPanel(B2.data(), N, ld, p2.data(), d2.data());
        bool same = o1 == o2;
        if (o1 && o2) same = same && memcmp(A.data(), B2.data(), A.size() * sizeof(MT)) == 0 && p1 == p2 && memcmp(d1.data(), d2.data(), N * 8) == 0;
        if (!same) { bad++; if (bad < 5) printf("mismatch trial %d N %d ok %d %d\n", t, N, o1, o2); }
    }
    return bad;
}
int main() {
    std::mt19937_64 g(7);
    int b64 = run<double>(g, 1500), b32 = run<float>(g, 1500);
    printf("double mismatches %d, float mismatches %d\n", b64, b32);
    return b64 + b32 != 0;
}
