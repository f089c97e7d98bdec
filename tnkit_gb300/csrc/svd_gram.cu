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
#include <cmath>
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

template <typename T> struct La;

template <typename T>
int sizes(int64_t R, int64_t C, Handles* h, Layout* L, int orth = 0) {
    // orth 0: the smaller Gram matrix; orth 1 / 2: the R x R / C x C one (see svd_gram_direct)
    const int64_t n = orth == 1 ? R : orth == 2 ? C : (R < C ? R : C);
    const int64_t m = orth ? (R < C ? R : C) : (R < C ? C : R);
    int lw_ev = 0, lw_qr = 0, lw_or = 0;
    if (La<T>::syevd_ws(h->sol, (int)n, &lw_ev) != CUSOLVER_STATUS_SUCCESS ||
        (!orth && (La<T>::geqrf_ws(h->sol, (int)m, (int)n, &lw_qr) != CUSOLVER_STATUS_SUCCESS ||
                   La<T>::orgqr_ws(h->sol, (int)m, (int)n, &lw_or) !=
                       CUSOLVER_STATUS_SUCCESS))) {
        tnk::set_error("svd_gram: cuSOLVER workspace query failed (R=%lld, C=%lld)",
                       (long long)R, (long long)C);
        return TNK_ERR_CUDA;
    }
    const int lw = std::max(lw_ev, std::max(lw_qr, lw_or));
    const size_t es = sizeof(T);
    size_t o = 0;
    L->G = o; o += up(es * n * n);
    L->Y = o; o += up(es * (orth ? R * C : m * n));
    L->w = o; o += up(es * n);
    L->tau = o; o += up(es * n);
    L->sign = o; o += up(es * n);
    L->perm = o; o += up(sizeof(int) * n);
    L->info = o; o += up(sizeof(int) * 4);
    L->work = o; o += up(es * (size_t)lw);
    L->total = o;
    return TNK_OK;
}

// Reverse the column order of an n x n column-major matrix in place (eigenvectors ascending ->
// descending).
template <typename T>
__global__ void flip_cols(T* __restrict__ A, int64_t n) {
    const int64_t total = n * (n / 2);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = e / n, r = e - j * n;
        const T a = A[j * n + r];
        A[j * n + r] = A[(n - 1 - j) * n + r];
        A[(n - 1 - j) * n + r] = a;
    }
}

// Output column j is column perm[j] of the column-major src (ld, `rows` rows), times
// sign[perm[j]] when sign is given; written row-major as rows x k (transpose = 0:
// dst[r * k + j]) or k x rows (transpose = 1: dst[j * rows + r]).
template <typename T>
__global__ void gather_cols(const T* __restrict__ src, int64_t ld, int64_t rows,
                            const int* __restrict__ perm, const T* __restrict__ sign, int64_t k,
                            T* __restrict__ dst, int transpose) {
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
        T v = src[(int64_t)p * ld + r];
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

// cuBLAS / cuSOLVER entry points by element type
template <> struct La<double> {
    static cublasStatus_t syrk(cublasHandle_t h, cublasOperation_t tr, int n, int k,
                               const double* A, int lda, double* C, int ldc) {
        const double one = 1.0, zero = 0.0;
        return cublasDsyrk(h, CUBLAS_FILL_MODE_LOWER, tr, n, k, &one, A, lda, &zero, C, ldc);
    }
    static cublasStatus_t gemm(cublasHandle_t h, cublasOperation_t ta, int m, int n, int k,
                               const double* A, int lda, const double* B, int ldb, double* C,
                               int ldc) {
        const double one = 1.0, zero = 0.0;
        return cublasDgemm(h, ta, CUBLAS_OP_N, m, n, k, &one, A, lda, B, ldb, &zero, C, ldc);
    }
    static cusolverStatus_t syevd_ws(cusolverDnHandle_t h, int n, int* lw) {
        return cusolverDnDsyevd_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                           n, nullptr, n, nullptr, lw);
    }
    static cusolverStatus_t geqrf_ws(cusolverDnHandle_t h, int m, int n, int* lw) {
        return cusolverDnDgeqrf_bufferSize(h, m, n, nullptr, m, lw);
    }
    static cusolverStatus_t orgqr_ws(cusolverDnHandle_t h, int m, int n, int* lw) {
        return cusolverDnDorgqr_bufferSize(h, m, n, n, nullptr, m, nullptr, lw);
    }
    static cusolverStatus_t syevd(cusolverDnHandle_t h, int n, double* A, double* w,
                                  double* work, int lw, int* info) {
        return cusolverDnDsyevd(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, A, n, w,
                                work, lw, info);
    }
    static cusolverStatus_t geqrf(cusolverDnHandle_t h, int m, int n, double* A, double* tau,
                                  double* work, int lw, int* info) {
        return cusolverDnDgeqrf(h, m, n, A, m, tau, work, lw, info);
    }
    static cusolverStatus_t orgqr(cusolverDnHandle_t h, int m, int n, double* A,
                                  const double* tau, double* work, int lw, int* info) {
        return cusolverDnDorgqr(h, m, n, n, A, m, tau, work, lw, info);
    }
};
template <> struct La<float> {
    static cublasStatus_t syrk(cublasHandle_t h, cublasOperation_t tr, int n, int k,
                               const float* A, int lda, float* C, int ldc) {
        const float one = 1.0f, zero = 0.0f;
        return cublasSsyrk(h, CUBLAS_FILL_MODE_LOWER, tr, n, k, &one, A, lda, &zero, C, ldc);
    }
    static cublasStatus_t gemm(cublasHandle_t h, cublasOperation_t ta, int m, int n, int k,
                               const float* A, int lda, const float* B, int ldb, float* C,
                               int ldc) {
        const float one = 1.0f, zero = 0.0f;
        return cublasSgemm(h, ta, CUBLAS_OP_N, m, n, k, &one, A, lda, B, ldb, &zero, C, ldc);
    }
    static cusolverStatus_t syevd_ws(cusolverDnHandle_t h, int n, int* lw) {
        return cusolverDnSsyevd_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                           n, nullptr, n, nullptr, lw);
    }
    static cusolverStatus_t geqrf_ws(cusolverDnHandle_t h, int m, int n, int* lw) {
        return cusolverDnSgeqrf_bufferSize(h, m, n, nullptr, m, lw);
    }
    static cusolverStatus_t orgqr_ws(cusolverDnHandle_t h, int m, int n, int* lw) {
        return cusolverDnSorgqr_bufferSize(h, m, n, n, nullptr, m, nullptr, lw);
    }
    static cusolverStatus_t syevd(cusolverDnHandle_t h, int n, float* A, float* w, float* work,
                                  int lw, int* info) {
        return cusolverDnSsyevd(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, A, n, w,
                                work, lw, info);
    }
    static cusolverStatus_t geqrf(cusolverDnHandle_t h, int m, int n, float* A, float* tau,
                                  float* work, int lw, int* info) {
        return cusolverDnSgeqrf(h, m, n, A, m, tau, work, lw, info);
    }
    static cusolverStatus_t orgqr(cusolverDnHandle_t h, int m, int n, float* A,
                                  const float* tau, float* work, int lw, int* info) {
        return cusolverDnSorgqr(h, m, n, n, A, m, tau, work, lw, info);
    }
};

}  // namespace

namespace {

template <typename T>
int svd_gram_ws(int64_t R, int64_t C, int64_t* bytes, int orth = 0) {
    if (R < 1 || C < 1 || !bytes || R * C > (int64_t)1 << 30 || orth < 0 || orth > 2) {
        tnk::set_error("svd_gram_ws: bad argument");
        return TNK_ERR_ARG;
    }
    Handles* h = nullptr;
    int rc = handles_for_current_device(&h);
    if (rc) return rc;
    Layout L;
    rc = sizes<T>(R, C, h, &L, orth);
    if (rc) return rc;
    *bytes = (int64_t)L.total;
    return TNK_OK;
}

// orth = 1: U orthonormal from the eigenvectors of M M^T, Vh = diag(1/S) U^T M; orth = 2: Vh
// orthonormal from the eigenvectors of M^T M, U = M V diag(1/S); S = sqrt(max(lambda, 0)) in
// descending order. No QR: the factor the sweep keeps canonical comes straight from its Gram
// matrix, the other carries S and is the exact projection.
template <typename T>
int svd_gram_direct(const T* M, int64_t R, int64_t C, T* U, T* S, T* Vh, char* base,
                    const Layout& L, Handles* h, int orth, double* S_host, cudaStream_t st) {
    T* G = reinterpret_cast<T*>(base + L.G);
    T* Y = reinterpret_cast<T*>(base + L.Y);
    T* w = reinterpret_cast<T*>(base + L.w);
    T* inv = reinterpret_cast<T*>(base + L.sign);
    int* perm = reinterpret_cast<int*>(base + L.perm);
    int* info = reinterpret_cast<int*>(base + L.info);
    T* work = reinterpret_cast<T*>(base + L.work);
    const int lwork = (int)((L.total - L.work) / sizeof(T));
    const int g = orth == 1 ? (int)R : (int)C;          // Gram order
    const int k = (int)(R < C ? R : C);                 // rank kept
    // X = M^T is C x R column-major (ld C): M M^T = X^T X, M^T M = X X^T
    int rc = check_blas(La<T>::syrk(h->blas, orth == 1 ? CUBLAS_OP_T : CUBLAS_OP_N, g,
                                    orth == 1 ? (int)C : (int)R, M, (int)C, G, g), "syrk");
    if (rc) return rc;
    if ((rc = check_sol(La<T>::syevd(h->sol, g, G, w, work, lwork, info), "syevd"))) return rc;
    const int threads = 256;
    auto blocks = [&](int64_t e) {
        int64_t b = (e + threads - 1) / threads;
        return (int)(b > 4096 ? 4096 : (b < 1 ? 1 : b));
    };
    flip_cols<T><<<blocks((int64_t)g * (g / 2)), threads, 0, st>>>(G, g);
    if ((rc = tnk::check_launch("flip_cols"))) return rc;
    // the other factor, unscaled: orth 1: Z = X U (C x k, ld C) = (U^T M)^T; orth 2: Y = X^T V
    // (R x k, ld R) = M V
    if (orth == 1)
        rc = check_blas(La<T>::gemm(h->blas, CUBLAS_OP_N, (int)C, k, (int)R, M, (int)C, G, g, Y,
                                    (int)C), "gemm");
    else
        rc = check_blas(La<T>::gemm(h->blas, CUBLAS_OP_T, (int)R, k, (int)C, M, (int)C, G, g, Y,
                                    (int)R), "gemm");
    if (rc) return rc;
    std::vector<T> lam(g);
    int hinfo = 0;
    if (cudaMemcpyAsync(lam.data(), w, sizeof(T) * g, cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        tnk::set_error("svd_gram: %s", cudaGetErrorString(cudaGetLastError()));
        return TNK_ERR_CUDA;
    }
    if (hinfo) {
        tnk::set_error("svd_gram: cuSOLVER info syevd=%d (R=%lld, C=%lld)", hinfo,
                       (long long)R, (long long)C);
        return TNK_ERR_CUDA;
    }
    std::vector<T> sv(k), iv(k);
    std::vector<int> id(k);
    for (int j = 0; j < k; ++j) {
        const T l = lam[g - 1 - j];
        sv[j] = l > 0 ? (T)std::sqrt((double)l) : (T)0;
        iv[j] = sv[j] > 0 ? (T)1 / sv[j] : (T)0;
        id[j] = j;
    }
    if (S_host)
        for (int j = 0; j < k; ++j) S_host[j] = (double)sv[j];
    if (cudaMemcpyAsync(perm, id.data(), sizeof(int) * k, cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(inv, iv.data(), sizeof(T) * k, cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(S, sv.data(), sizeof(T) * k, cudaMemcpyHostToDevice, st) !=
            cudaSuccess) {
        tnk::set_error("svd_gram: upload of the scales failed");
        return TNK_ERR_CUDA;
    }
    if (orth == 1) {
        // U = eigenvectors (R x k row-major); Vh[j, c] = Z[c + j C] / S_j
        gather_cols<T><<<blocks((int64_t)R * k), threads, 0, st>>>(G, g, R, perm, nullptr, k, U,
                                                                   0);
        gather_cols<T><<<blocks((int64_t)C * k), threads, 0, st>>>(Y, C, C, perm, inv, k, Vh,
                                                                   1);
    } else {
        // U[r, j] = Y[r + j R] / S_j; Vh = V^T (k x C row-major)
        gather_cols<T><<<blocks((int64_t)R * k), threads, 0, st>>>(Y, R, R, perm, inv, k, U, 0);
        gather_cols<T><<<blocks((int64_t)C * k), threads, 0, st>>>(G, g, C, perm, nullptr, k,
                                                                   Vh, 1);
    }
    rc = tnk::check_launch("gather_cols");
    if (rc) return rc;
    if (cudaStreamSynchronize(st) != cudaSuccess) {
        tnk::set_error("svd_gram: %s", cudaGetErrorString(cudaGetLastError()));
        return TNK_ERR_CUDA;
    }
    return TNK_OK;
}

template <typename T>
int svd_gram(const T* M, int64_t R, int64_t C, T* U, T* S, T* Vh, void* ws, int64_t ws_bytes,
             double* S_host, cudaStream_t st, int orth = 0) {
    if (!M || !U || !S || !Vh || !ws || R < 1 || C < 1 || R * C > (int64_t)1 << 30 || orth < 0 ||
        orth > 2) {
        tnk::set_error("svd_gram: bad argument");
        return TNK_ERR_ARG;
    }
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
    rc = sizes<T>(R, C, h, &L, orth);
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
    if (orth == 1 || orth == 2)
        return svd_gram_direct<T>(M, R, C, U, S, Vh, base, L, h, orth, S_host, st);
    T* G = reinterpret_cast<T*>(base + L.G);
    T* Y = reinterpret_cast<T*>(base + L.Y);
    T* w = reinterpret_cast<T*>(base + L.w);
    T* tau = reinterpret_cast<T*>(base + L.tau);
    T* sgn = reinterpret_cast<T*>(base + L.sign);
    int* perm = reinterpret_cast<int*>(base + L.perm);
    int* info = reinterpret_cast<int*>(base + L.info);
    T* work = reinterpret_cast<T*>(base + L.work);
    const int lwork = (int)((L.total - L.work) / sizeof(T));
    const bool tall = R >= C;
    const int n = (int)(tall ? C : R), m = (int)(tall ? R : C);
    // X = M^T is C x R column-major (ld C): G = M^T M = X X^T (tall) or M M^T = X^T X (wide)
    rc = check_blas(La<T>::syrk(h->blas, tall ? CUBLAS_OP_N : CUBLAS_OP_T, n,
                                (int)(tall ? R : C), M, (int)C, G, n), "syrk");
    if (rc) return rc;
    if ((rc = check_sol(La<T>::syevd(h->sol, n, G, w, work, lwork, info), "syevd"))) return rc;
    const int threads = 256;
    auto blocks = [&](int64_t e) {
        int64_t b = (e + threads - 1) / threads;
        return (int)(b > 4096 ? 4096 : (b < 1 ? 1 : b));
    };
    // eigenvectors in descending order of the eigenvalue
    flip_cols<T><<<blocks((int64_t)n * (n / 2)), threads, 0, st>>>(G, n);
    if ((rc = tnk::check_launch("flip_cols"))) return rc;
    // Y = M V (R x C, tall) or M^T U (C x R, wide), column-major with ld m
    rc = check_blas(La<T>::gemm(h->blas, tall ? CUBLAS_OP_T : CUBLAS_OP_N, m, n, n, M, (int)C,
                                G, n, Y, m), "gemm");
    if (rc) return rc;
    if ((rc = check_sol(La<T>::geqrf(h->sol, m, n, Y, tau, work, lwork, info + 1), "geqrf")))
        return rc;
    // d = diag(R) to the host (the sort happens there)
    std::vector<T> d(n);
    if (cudaMemcpy2DAsync(d.data(), sizeof(T), Y, sizeof(T) * (m + 1), sizeof(T), n,
                          cudaMemcpyDeviceToHost, st) != cudaSuccess) {
        tnk::set_error("svd_gram: diagonal copy failed");
        return TNK_ERR_CUDA;
    }
    if ((rc = check_sol(La<T>::orgqr(h->sol, m, n, Y, tau, work, lwork, info + 2), "orgqr")))
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
    std::vector<T> sv(n), sg(n);
    for (int j = 0; j < n; ++j) {
        sv[j] = d[j] < 0 ? -d[j] : d[j];
        sg[j] = sv[j] > 0 ? d[j] / sv[j] : (T)1;
    }
    std::vector<int> o(n);
    std::iota(o.begin(), o.end(), 0);
    std::stable_sort(o.begin(), o.end(), [&](int a, int b) { return sv[a] > sv[b]; });
    std::vector<T> so(n);
    for (int j = 0; j < n; ++j) so[j] = sv[o[j]];
    if (S_host)
        for (int j = 0; j < n; ++j) S_host[j] = (double)so[j];
    if (cudaMemcpyAsync(perm, o.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(sgn, sg.data(), sizeof(T) * n, cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(S, so.data(), sizeof(T) * n, cudaMemcpyHostToDevice, st) !=
            cudaSuccess) {
        tnk::set_error("svd_gram: upload of the order failed");
        return TNK_ERR_CUDA;
    }
    if (tall) {
        // U = Q[:, o] * sign (R x n row-major); Vh = (V flipped)[:, o]^T (n x C row-major)
        gather_cols<T><<<blocks((int64_t)R * n), threads, 0, st>>>(Y, m, R, perm, sgn, n, U, 0);
        gather_cols<T><<<blocks((int64_t)C * n), threads, 0, st>>>(G, n, C, perm, nullptr, n,
                                                                   Vh, 1);
    } else {
        // U = (U flipped)[:, o] (R x n row-major); Vh = (Q[:, o] * sign)^T (n x C row-major)
        gather_cols<T><<<blocks((int64_t)R * n), threads, 0, st>>>(G, n, R, perm, nullptr, n, U,
                                                                   0);
        gather_cols<T><<<blocks((int64_t)C * n), threads, 0, st>>>(Y, m, C, perm, sgn, n, Vh,
                                                                   1);
    }
    rc = tnk::check_launch("gather_cols");
    if (rc) return rc;
    if (cudaStreamSynchronize(st) != cudaSuccess) {
        tnk::set_error("svd_gram: %s", cudaGetErrorString(cudaGetLastError()));
        return TNK_ERR_CUDA;
    }
    return TNK_OK;
}

}  // namespace

extern "C" int tnk_svd_gram_ws_f64(int64_t R, int64_t C, int64_t* bytes) {
    return svd_gram_ws<double>(R, C, bytes);
}

extern "C" int tnk_svd_gram_f64(const double* M, int64_t R, int64_t C, double* U, double* S,
                                double* Vh, void* ws, int64_t ws_bytes, double* S_host,
                                void* stream) {
    return svd_gram<double>(M, R, C, U, S, Vh, ws, ws_bytes, S_host, (cudaStream_t)stream);
}

extern "C" int tnk_svd_gram_ws_f32(int64_t R, int64_t C, int64_t* bytes) {
    return svd_gram_ws<float>(R, C, bytes);
}

extern "C" int tnk_svd_gram_f32(const float* M, int64_t R, int64_t C, float* U, float* S,
                                float* Vh, void* ws, int64_t ws_bytes, double* S_host,
                                void* stream) {
    return svd_gram<float>(M, R, C, U, S, Vh, ws, ws_bytes, S_host, (cudaStream_t)stream);
}

extern "C" int tnk_svd_gram_ws2_f64(int64_t R, int64_t C, int32_t orth, int64_t* bytes) {
    return svd_gram_ws<double>(R, C, bytes, orth);
}

extern "C" int tnk_svd_gram2_f64(const double* M, int64_t R, int64_t C, int32_t orth, double* U,
                                 double* S, double* Vh, void* ws, int64_t ws_bytes,
                                 double* S_host, void* stream) {
    return svd_gram<double>(M, R, C, U, S, Vh, ws, ws_bytes, S_host, (cudaStream_t)stream, orth);
}
