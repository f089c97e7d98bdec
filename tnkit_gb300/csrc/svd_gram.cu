// Per-sector factorisation of the DMRG truncation: U, S, Vh of one real block through the smaller
// Gram matrix -- the reference's method='gram' (tnkit/blocks.py:1345-1377): Hermitian eigh of
// M^T M (or M M^T), eigenvectors in descending order, a QR of M V (or M^T U) that
// re-orthonormalises the other factor, S = |diag R| with the signs moved into Q, and a
// descending stable sort by S.
//
// One call factors one block and returns when its outputs are written (it synchronises its
// stream: cuSOLVER's syevd waits on the host inside the call anyway). The Python side issues
// the sectors of a bond from a thread pool, one stream each; the call holds no interpreter
// lock, so the sectors overlap. cuBLAS/cuSOLVER handles are per host thread and device.
//
// Layouts: M is row-major R x C (the canonical block); U is written row-major R x k, Vh
// row-major k x C, S (k) descending, k = min(R, C). In cuBLAS's column-major view the block
// buffer is X = M^T (C x R, ld C).
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "tnk_internal.cuh"

namespace {

struct Handles {
    cublasHandle_t blas = nullptr;
    cusolverDnHandle_t sol = nullptr;
    int device = -1;
};

thread_local Handles g_h;

int handles_for_current_device(Handles** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        tnk::set_error("svd_gram: cudaGetDevice failed");
        return TNK_ERR_DEVICE;
    }
    if (g_h.device != dev) {
        if (g_h.blas) cublasDestroy(g_h.blas);
        if (g_h.sol) cusolverDnDestroy(g_h.sol);
        g_h = Handles{};
        if (cublasCreate(&g_h.blas) != CUBLAS_STATUS_SUCCESS ||
            cusolverDnCreate(&g_h.sol) != CUSOLVER_STATUS_SUCCESS) {
            tnk::set_error("svd_gram: cannot create cuBLAS/cuSOLVER handles on device %d", dev);
            return TNK_ERR_CUDA;
        }
        g_h.device = dev;
    }
    *out = &g_h;
    return TNK_OK;
}

// Workspace carve-up (bytes, 256-aligned pieces): G (n x n), Y (m x n), w (n), tau (n),
// d (n, host-sorted later), perm (n int32), sign (n), info (int32), cuSOLVER work.
struct Layout {
    size_t G, Y, w, tau, sign, perm, info, work, total;
};

inline size_t up(size_t x) { return (x + 255) & ~size_t(255); }

int sizes(int64_t R, int64_t C, Handles* h, Layout* L) {
    const int64_t n = R < C ? R : C, m = R < C ? C : R;
    int lw_ev = 0, lw_qr = 0, lw_or = 0;
    if (cusolverDnDsyevd_bufferSize(h->sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                    (int)n, nullptr, (int)n, nullptr, &lw_ev) !=
            CUSOLVER_STATUS_SUCCESS ||
        cusolverDnDgeqrf_bufferSize(h->sol, (int)m, (int)n, nullptr, (int)m, &lw_qr) !=
            CUSOLVER_STATUS_SUCCESS ||
        cusolverDnDorgqr_bufferSize(h->sol, (int)m, (int)n, (int)n, nullptr, (int)m, nullptr,
                                    &lw_or) != CUSOLVER_STATUS_SUCCESS) {
        tnk::set_error("svd_gram: cuSOLVER workspace query failed (R=%lld, C=%lld)",
                       (long long)R, (long long)C);
        return TNK_ERR_CUDA;
    }
    int lw = std::max(lw_ev, std::max(lw_qr, lw_or));
    size_t o = 0;
    L->G = o; o += up(sizeof(double) * n * n);
    L->Y = o; o += up(sizeof(double) * m * n);
    L->w = o; o += up(sizeof(double) * n);
    L->tau = o; o += up(sizeof(double) * n);
    L->sign = o; o += up(sizeof(double) * n);
    L->perm = o; o += up(sizeof(int) * n);
    L->info = o; o += up(sizeof(int) * 4);
    L->work = o; o += up(sizeof(double) * (size_t)lw);
    L->total = o;
    return TNK_OK;
}

// Reverse the column order of an n x n column-major matrix in place (eigenvectors ascending ->
// descending).
__global__ void flip_cols(double* __restrict__ A, int64_t n) {
    const int64_t total = n * (n / 2);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = e / n, r = e - j * n;
        const double a = A[j * n + r];
        A[j * n + r] = A[(n - 1 - j) * n + r];
        A[(n - 1 - j) * n + r] = a;
    }
}

// Output column j is column perm[j] of the column-major src (ld, `rows` rows), times
// sign[perm[j]] when sign is given; written row-major as rows x k (transpose = 0:
// dst[r * k + j]) or k x rows (transpose = 1: dst[j * rows + r]).
__global__ void gather_cols(const double* __restrict__ src, int64_t ld, int64_t rows,
                            const int* __restrict__ perm, const double* __restrict__ sign,
                            int64_t k, double* __restrict__ dst, int transpose) {
    const int64_t total = rows * k;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        int64_t r, j;
        if (transpose) {
            j = e / rows;
            r = e - j * rows;
        } else {
            r = e / k;
            j = e - r * k;
        }
        const int p = perm[j];
        double v = src[(int64_t)p * ld + r];
        if (sign) v *= sign[p];
        dst[e] = v;
    }
}

int check_blas(cublasStatus_t s, const char* what) {
    if (s != CUBLAS_STATUS_SUCCESS) {
        tnk::set_error("svd_gram: %s failed (cuBLAS status %d)", what, (int)s);
        return TNK_ERR_CUDA;
    }
    return TNK_OK;
}

int check_sol(cusolverStatus_t s, const char* what) {
    if (s != CUSOLVER_STATUS_SUCCESS) {
        tnk::set_error("svd_gram: %s failed (cuSOLVER status %d)", what, (int)s);
        return TNK_ERR_CUDA;
    }
    return TNK_OK;
}

}  // namespace

extern "C" int tnk_svd_gram_ws_f64(int64_t R, int64_t C, int64_t* bytes) {
    if (R < 1 || C < 1 || !bytes || R * C > (int64_t)1 << 30) {
        tnk::set_error("svd_gram_ws: bad argument");
        return TNK_ERR_ARG;
    }
    Handles* h = nullptr;
    int rc = handles_for_current_device(&h);
    if (rc) return rc;
    Layout L;
    rc = sizes(R, C, h, &L);
    if (rc) return rc;
    *bytes = (int64_t)L.total;
    return TNK_OK;
}

extern "C" int tnk_svd_gram_f64(const double* M, int64_t R, int64_t C, double* U, double* S,
                                double* Vh, void* ws, int64_t ws_bytes, double* S_host,
                                void* stream) {
    if (!M || !U || !S || !Vh || !ws || R < 1 || C < 1 || R * C > (int64_t)1 << 30) {
        tnk::set_error("svd_gram: bad argument");
        return TNK_ERR_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, M) != cudaSuccess || pa.type != cudaMemoryTypeDevice) {
        tnk::set_error("svd_gram: M is not device memory");
        return TNK_ERR_ARG;
    }
    if (cudaSetDevice(pa.device) != cudaSuccess) {
        tnk::set_error("svd_gram: cudaSetDevice(%d) failed", pa.device);
        return TNK_ERR_DEVICE;
    }
    Handles* h = nullptr;
    int rc = handles_for_current_device(&h);
    if (rc) return rc;
    Layout L;
    rc = sizes(R, C, h, &L);
    if (rc) return rc;
    if (ws_bytes < (int64_t)L.total || ((uintptr_t)ws & 255)) {
        tnk::set_error("svd_gram: workspace of %lld bytes (256-aligned) needed, got %lld",
                       (long long)L.total, (long long)ws_bytes);
        return TNK_ERR_SIZE;
    }
    if ((rc = check_blas(cublasSetStream(h->blas, st), "cublasSetStream")) ||
        (rc = check_sol(cusolverDnSetStream(h->sol, st), "cusolverDnSetStream")))
        return rc;
    char* base = static_cast<char*>(ws);
    double* G = reinterpret_cast<double*>(base + L.G);
    double* Y = reinterpret_cast<double*>(base + L.Y);
    double* w = reinterpret_cast<double*>(base + L.w);
    double* tau = reinterpret_cast<double*>(base + L.tau);
    double* sgn = reinterpret_cast<double*>(base + L.sign);
    int* perm = reinterpret_cast<int*>(base + L.perm);
    int* info = reinterpret_cast<int*>(base + L.info);
    double* work = reinterpret_cast<double*>(base + L.work);
    const int lwork = (int)((L.total - L.work) / sizeof(double));
    const bool tall = R >= C;
    const int n = (int)(tall ? C : R), m = (int)(tall ? R : C);
    const double one = 1.0, zero = 0.0;
    // X = M^T is C x R column-major (ld C)
    if (tall) {
        // G = M^T M = X X^T (C x C); Y = M V = X^T V (R x C, ld R)
        rc = check_blas(cublasDsyrk(h->blas, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, n, (int)R,
                                    &one, M, (int)C, &zero, G, n), "syrk");
    } else {
        // G = M M^T = X^T X (R x R); Y = M^T U = X U (C x R, ld C)
        rc = check_blas(cublasDsyrk(h->blas, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, n, (int)C,
                                    &one, M, (int)C, &zero, G, n), "syrk");
    }
    if (rc) return rc;
    if ((rc = check_sol(cusolverDnDsyevd(h->sol, CUSOLVER_EIG_MODE_VECTOR,
                                         CUBLAS_FILL_MODE_LOWER, n, G, n, w, work, lwork, info),
                        "syevd")))
        return rc;
    const int threads = 256;
    auto blocks = [&](int64_t e) {
        int64_t b = (e + threads - 1) / threads;
        return (int)(b > 4096 ? 4096 : (b < 1 ? 1 : b));
    };
    // eigenvectors in descending order of the eigenvalue
    flip_cols<<<blocks((int64_t)n * (n / 2)), threads, 0, st>>>(G, n);
    if ((rc = tnk::check_launch("flip_cols"))) return rc;
    // Y = M V (R x C, tall) or M^T U (C x R, wide), column-major with ld m
    if (tall)
        rc = check_blas(cublasDgemm(h->blas, CUBLAS_OP_T, CUBLAS_OP_N, m, n, n, &one, M,
                                    (int)C, G, n, &zero, Y, m), "gemm");
    else
        rc = check_blas(cublasDgemm(h->blas, CUBLAS_OP_N, CUBLAS_OP_N, m, n, n, &one, M,
                                    (int)C, G, n, &zero, Y, m), "gemm");
    if (rc) return rc;
    if ((rc = check_sol(cusolverDnDgeqrf(h->sol, m, n, Y, m, tau, work, lwork, info + 1),
                        "geqrf")))
        return rc;
    // d = diag(R) to the host (the sort happens there)
    std::vector<double> d(n), s(n), sg(n);
    if (cudaMemcpy2DAsync(d.data(), sizeof(double), Y, sizeof(double) * (m + 1), sizeof(double),
                          n, cudaMemcpyDeviceToHost, st) != cudaSuccess) {
        tnk::set_error("svd_gram: diagonal copy failed");
        return TNK_ERR_CUDA;
    }
    if ((rc = check_sol(cusolverDnDorgqr(h->sol, m, n, n, Y, m, tau, work, lwork, info + 2),
                        "orgqr")))
        return rc;
    int hinfo[3] = {0, 0, 0};
    if (cudaMemcpyAsync(hinfo, info, sizeof(hinfo), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        tnk::set_error("svd_gram: %s", cudaGetErrorString(cudaGetLastError()));
        return TNK_ERR_CUDA;
    }
    if (hinfo[0] || hinfo[1] || hinfo[2]) {
        tnk::set_error("svd_gram: cuSOLVER info syevd=%d geqrf=%d orgqr=%d (R=%lld, C=%lld)",
                       hinfo[0], hinfo[1], hinfo[2], (long long)R, (long long)C);
        return TNK_ERR_CUDA;
    }
    for (int j = 0; j < n; ++j) {
        s[j] = d[j] < 0 ? -d[j] : d[j];
        sg[j] = s[j] > 0 ? d[j] / s[j] : 1.0;
    }
    std::vector<int> o(n);
    std::iota(o.begin(), o.end(), 0);
    std::stable_sort(o.begin(), o.end(), [&](int a, int b) { return s[a] > s[b]; });
    std::vector<double> so(n);
    for (int j = 0; j < n; ++j) so[j] = s[o[j]];
    if (S_host) std::copy(so.begin(), so.end(), S_host);
    if (cudaMemcpyAsync(perm, o.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(sgn, sg.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(S, so.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st) !=
            cudaSuccess) {
        tnk::set_error("svd_gram: upload of the order failed");
        return TNK_ERR_CUDA;
    }
    if (tall) {
        // U = Q[:, o] * sign (R x n row-major); Vh = (V flipped)[:, o]^T (n x C row-major)
        gather_cols<<<blocks((int64_t)R * n), threads, 0, st>>>(Y, m, R, perm, sgn, n, U, 0);
        gather_cols<<<blocks((int64_t)C * n), threads, 0, st>>>(G, n, C, perm, nullptr, n, Vh,
                                                                1);
    } else {
        // U = (U flipped)[:, o] (R x n row-major); Vh = (Q[:, o] * sign)^T (n x C row-major)
        gather_cols<<<blocks((int64_t)R * n), threads, 0, st>>>(G, n, R, perm, nullptr, n, U,
                                                                0);
        gather_cols<<<blocks((int64_t)C * n), threads, 0, st>>>(Y, m, C, perm, sgn, n, Vh, 1);
    }
    rc = tnk::check_launch("gather_cols");
    if (rc) return rc;
    if (cudaStreamSynchronize(st) != cudaSuccess) {
        tnk::set_error("svd_gram: %s", cudaGetErrorString(cudaGetLastError()));
        return TNK_ERR_CUDA;
    }
    return TNK_OK;
}
