// Non-reversible models: the complex eigen system of Q as the engine keeps it
// (d_nr), and P(t) and its time derivatives built from it, shared by the
// mixed-precision and FP64 precompute and branch kernels.
#pragma once
#include <cuda_runtime.h>

namespace iqg {

struct NonrevModel {
    const double *er, *ei, *vr, *vi, *wr, *wi, *root, *tipv;  // ceval, cevec, cinv_evec (re, im), root freq, tip vectors
};
__host__ __device__ inline NonrevModel nonrev_model(const double *nr, int n, int S) {
    const long long nn = (long long)n * n;
    NonrevModel m;
    m.er = nr;
    m.ei = nr + n;
    m.vr = nr + 2 * n;
    m.vi = m.vr + nn;
    m.wr = m.vi + nn;
    m.wi = m.wr + nn;
    m.root = m.wi + nn;
    m.tipv = m.root + n;
    (void)S;
    return m;
}

// out[x][y] = Re(sum_i V[x][i] (lambda_i r)^k exp(lambda_i r t) V^-1[i][y]) for
// x, y < n, FP64, into shared memory (n*n doubles); e holds 2n doubles of scratch.
__device__ inline void nonrev_matrix(const NonrevModel &m, int n, double r, double t, int k, double *e, double *out) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double a = m.er[i] * r, b = m.ei[i] * r;  // lambda_i r
        const double g = exp(a * t);
        double re = g * cos(b * t), im = g * sin(b * t);
        for (int j = 0; j < k; j++) {  // times (lambda_i r)^k
            const double nr = re * a - im * b, ni = re * b + im * a;
            re = nr;
            im = ni;
        }
        e[i] = re;
        e[n + i] = im;
    }
    __syncthreads();
    for (int t2 = threadIdx.x; t2 < n * n; t2 += blockDim.x) {
        const int x = t2 / n, y = t2 % n;
        double acc = 0.0;
        for (int i = 0; i < n; i++) {
            // (V[x][i] * E_i) * W[i][y], real part
            const double pr = m.vr[x * n + i] * e[i] - m.vi[x * n + i] * e[n + i];
            const double pi = m.vr[x * n + i] * e[n + i] + m.vi[x * n + i] * e[i];
            acc = fma(pr, m.wr[i * n + y], acc);
            acc = fma(-pi, m.wi[i * n + y], acc);
        }
        out[t2] = acc;
    }
    __syncthreads();
}

}  // namespace iqg
