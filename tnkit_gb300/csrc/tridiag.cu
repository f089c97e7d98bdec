// Eigenvalues and eigenvectors of small real symmetric tridiagonal matrices on the GPU: the
// projected problems of the Krylov solvers (the Lanczos tridiagonal of the TDVP exponential,
// order <= a few dozen), solved where their coefficients were computed instead of on the host.
//
// Method: the implicit QL algorithm with a Wilkinson-type shift (Bowdler, Martin, Reinsch and
// Wilkinson, "The QR and QL algorithms for symmetric matrices", Numer. Math. 11 (1968) 293;
// Golub and Van Loan, Matrix Computations, section 8.3). An unreduced block [l, m] is found by
// the negligibility test |e_i| <= eps (|d_i| + |d_i+1|); one implicit QL step chases the shift's
// bulge from the bottom of the block up with Givens rotations; each rotation is recorded, and
// after the step every thread applies the step's rotations, in order, to its own row of the
// eigenvector matrix (so the serial part is only the O(m) rotation chain, and the O(n m) update
// runs n-wide without a barrier per rotation). At most TNK_TRIDIAG_MAX_ITER steps per
// eigenvalue; a matrix that needs more gets a positive info (the index of the eigenvalue that
// did not converge, as LAPACK's steqr reports it) and its outputs are left as they stand.
// Eigenvalues come out ascending with their vectors (columns of V).
//
// One thread block per matrix, threads = rows; shared memory holds the matrix's eigenvector
// rows (odd row stride: no bank conflicts when every thread reads its row's column i), the
// diagonal, the off-diagonal and one step's rotations.
#include <math.h>

#include "tnk_internal.cuh"

#define TNK_TRIDIAG_MAX_ITER 60

namespace {

__device__ __forceinline__ double sgn_of(double a, double b) {
    return b >= 0.0 ? fabs(a) : -fabs(a);
}

__global__ void tridiag_ql_kernel(const double* __restrict__ d_in, const double* __restrict__ e_in,
                                  int n, int64_t ld_d, int64_t ld_e, double* __restrict__ lam,
                                  double* __restrict__ V, int32_t* __restrict__ info) {
    extern __shared__ double sh[];
    const int zs = n | 1;                       // odd row stride of Z
    double* Z = sh;                             // n x zs
    double* d = Z + (size_t)n * zs;             // n
    double* e = d + n;                          // n (e[n-1] = 0)
    double* rc = e + n;                         // n: cosines of one step
    double* rs = rc + n;                        // n: sines of one step
    __shared__ int s_l, s_lo, s_hi, s_fail, s_go;

    const int b = blockIdx.x;
    const int t = threadIdx.x;
    for (int i = t; i < n; i += blockDim.x) {
        d[i] = d_in[b * ld_d + i];
        e[i] = (i < n - 1) ? e_in[b * ld_e + i] : 0.0;
        for (int j = 0; j < n; ++j) Z[i * zs + j] = (i == j) ? 1.0 : 0.0;
    }
    if (t == 0) {
        s_l = 0;
        s_fail = 0;
    }
    __syncthreads();

    int iters = 0;
    while (true) {
        if (t == 0) {
            // find the next unreduced block starting at l
            int l = s_l;
            s_go = 0;
            while (l < n) {
                int m = l;
                while (m < n - 1) {
                    double dd = fabs(d[m]) + fabs(d[m + 1]);
                    if (fabs(e[m]) <= 2.220446049250313e-16 * dd) break;
                    ++m;
                }
                if (m == l) {
                    ++l;                        // d[l] is an eigenvalue
                    iters = 0;
                    continue;
                }
                if (++iters > TNK_TRIDIAG_MAX_ITER) {
                    s_fail = l + 1;
                    break;
                }
                // one implicit QL step on [l, m] with the shift from the leading 2 x 2 block
                double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
                double r = hypot(g, 1.0);
                g = d[m] - d[l] + e[l] / (g + sgn_of(r, g));
                double s = 1.0, c = 1.0, p = 0.0;
                int i = m - 1;
                bool under = false;
                for (; i >= l; --i) {
                    double f = s * e[i];
                    double bb = c * e[i];
                    r = hypot(f, g);
                    e[i + 1] = r;
                    if (r == 0.0) {             // exact underflow: the block splits at i + 1
                        d[i + 1] -= p;
                        e[m] = 0.0;
                        under = true;
                        break;
                    }
                    s = f / r;
                    c = g / r;
                    g = d[i + 1] - p;
                    r = (d[i] - g) * s + 2.0 * c * bb;
                    p = s * r;
                    d[i + 1] = g + p;
                    g = c * r - bb;
                    rc[i] = c;
                    rs[i] = s;
                }
                if (!under) {
                    d[l] -= p;
                    e[l] = g;
                    e[m] = 0.0;
                    s_lo = l;
                } else {
                    s_lo = i + 1;               // rotations recorded for i+1 .. m-1 only
                }
                s_hi = m - 1;
                s_go = 1;
                break;
            }
            s_l = l;
        }
        __syncthreads();
        if (!s_go) break;                       // all eigenvalues found, or a failure
        // apply the step's rotations (i = hi down to lo) to every row of Z
        const int lo = s_lo, hi = s_hi;
        for (int k = t; k < n; k += blockDim.x) {
            double* zk = Z + (size_t)k * zs;
            for (int i = hi; i >= lo; --i) {
                const double c = rc[i], s = rs[i];
                const double f = zk[i + 1];
                zk[i + 1] = s * zk[i] + c * f;
                zk[i] = c * zk[i] - s * f;
            }
        }
        __syncthreads();
    }
    // ascending order: each eigenvalue's rank (ties by index), then scatter values and columns
    for (int j = t; j < n; j += blockDim.x) {
        int rank = 0;
        const double v = d[j];
        for (int q = 0; q < n; ++q) rank += (d[q] < v) || (d[q] == v && q < j);
        lam[b * (int64_t)n + rank] = v;
        for (int i = 0; i < n; ++i) V[(b * (int64_t)n + i) * n + rank] = Z[i * zs + j];
    }
    if (t == 0) info[b] = s_fail;
}

}  // namespace

extern "C" int tnk_tridiag_eig_f64(const double* d, const double* e, int64_t n, int64_t batch,
                                   int64_t ld_d, int64_t ld_e, double* lam, double* V,
                                   int32_t* info, void* stream) {
    if (n < 1 || n > TNK_TRIDIAG_MAX_N || batch < 0 || batch > 2147483647LL) {
        tnk::set_error("tridiag_eig: order %lld outside [1, %d] or bad batch %lld",
                       (long long)n, TNK_TRIDIAG_MAX_N, (long long)batch);
        return TNK_ERR_ARG;
    }
    if (ld_d < n || (n > 1 && ld_e < n - 1)) {
        tnk::set_error("tridiag_eig: leading dimensions %lld, %lld below the order %lld",
                       (long long)ld_d, (long long)ld_e, (long long)n);
        return TNK_ERR_ARG;
    }
    if (batch == 0) return TNK_OK;
    if (!d || (n > 1 && !e) || !lam || !V || !info) {
        tnk::set_error("tridiag_eig: null pointer");
        return TNK_ERR_ARG;
    }
    const int nn = (int)n;
    const size_t smem = ((size_t)nn * (nn | 1) + 4 * (size_t)nn) * sizeof(double);
    // the opt-in shared memory size is a per-device function attribute: set it once per device
    static bool attr_set[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        tnk::set_error("tridiag_eig: no usable current device");
        return TNK_ERR_DEVICE;
    }
    if (!attr_set[dev]) {
        cudaError_t a = cudaFuncSetAttribute(tridiag_ql_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)((TNK_TRIDIAG_MAX_N * (TNK_TRIDIAG_MAX_N | 1) +
                                                    4 * TNK_TRIDIAG_MAX_N) * sizeof(double)));
        if (a != cudaSuccess) {
            tnk::set_error("tridiag_eig: shared memory attribute: %s", cudaGetErrorString(a));
            return TNK_ERR_CUDA;
        }
        attr_set[dev] = true;
    }
    const int threads = nn <= 32 ? 32 : (nn <= 64 ? 64 : 128);
    tridiag_ql_kernel<<<(unsigned)batch, threads, smem, (cudaStream_t)stream>>>(
        d, n > 1 ? e : d, nn, ld_d, n > 1 ? ld_e : 0, lam, V, info);
    return tnk::check_launch("tridiag_eig");
}
