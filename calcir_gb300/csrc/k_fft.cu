// Lineshape transform: the unnormalised inverse real DFT of the zero-padded TCF with
// cuFFT's C2R convention (calcIR.cu:790-825): only X_0..X_{n/2} are read, Im X_0 (and
// Im X_{n/2} for even n) is ignored, and y_k = sum_j Z_j exp(+2 pi i j k / n) over the
// Hermitian extension Z.  n = ntcfpoints + nzeros is not a power of two (25750 =
// 2 * 5^3 * 103 by default), so this is a self-sorting mixed-radix Stockham FFT with one
// pass per prime factor; each output of a radix-p pass is a p-term sum
//     out[k' + L' j'] = sum_q exp(+2 pi i q k'/L') in[(k' mod L) + L (j' + r' q)],
// L' = L p, r' = n / L'.  The transform runs once per job, in double precision.
#include "cir_device.cuh"
#include <vector>

namespace {

__global__ void k_hermitian(const double *X, int nx, int n, double2 *Z) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int src = j <= n / 2 ? j : n - j;
    double re = 0, im = 0;
    if (src < nx) { re = X[2 * src]; im = X[2 * src + 1]; }
    if (src == 0 || (2 * src == n)) im = 0;
    if (j > n / 2) im = -im;
    Z[j] = make_double2(re, im);
}

__global__ void k_stockham(const double2 *in, double2 *out, int n, int L, int p) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n) return;
    const int Lp = L * p, rp = n / Lp;
    const int kp = idx % Lp, jp = idx / Lp, k = kp % L;
    double re = 0, im = 0;
    for (int q = 0; q < p; q++) {
        const long long ph = ((long long)q * kp) % Lp;
        double s, c;
        sincospi(2.0 * (double)ph / (double)Lp, &s, &c);
        const double2 v = in[k + (size_t)L * (jp + (size_t)rp * q)];
        re += c * v.x - s * v.y;
        im += c * v.y + s * v.x;
    }
    out[idx] = make_double2(re, im);
}

__global__ void k_realpart(const double2 *z, int n, double *y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = z[i].x;
}

}  // namespace

cudaError_t cir_launch_c2r(const double *X, int nx, int n, double *work0, double *work1, double *y, cudaStream_t s,
                           int *launches) {
    double2 *a = reinterpret_cast<double2 *>(work0), *b = reinterpret_cast<double2 *>(work1);
    const int T = 256, G = (n + T - 1) / T;
    k_hermitian<<<G, T, 0, s>>>(X, nx, n, a);
    int cnt = 1;
    std::vector<int> fac;
    int m = n;
    for (int p = 2; (long long)p * p <= m; p++)
        while (m % p == 0) { fac.push_back(p); m /= p; }
    if (m > 1) fac.push_back(m);
    int L = 1;
    for (int p : fac) {
        k_stockham<<<G, T, 0, s>>>(a, b, n, L, p);
        cnt++;
        double2 *t = a; a = b; b = t;
        L *= p;
    }
    k_realpart<<<G, T, 0, s>>>(a, n, y);
    cnt++;
    if (launches) *launches += cnt;
    return cudaGetLastError();
}
