// Lanczos vector kernels (FP64, sm_103a): dot, norm, the two GEMV passes of classical
// Gram-Schmidt, and scalar updates that read their scalars from device memory.
//
// All are HBM-bound streams. Reductions are two-phase and deterministic: phase 1 writes one
// partial per CTA (warp-shuffle, then shared-memory reduction), phase 2 sums the partials in a
// fixed order in one CTA. Grids are multiples of the 152 SMs, capped so the partials fit the
// caller's TNK_RED_ELEMS workspace.
#include "tnk_internal.cuh"

namespace tnk {
namespace {

constexpr int NT = 256;
constexpr int NSM = 152;
constexpr int MAXNV = 64;
constexpr int MD_ROWS = 8;   // rows of V reduced per pass of the multidot kernel

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum; result valid in thread 0. `sh` holds NT/32 doubles.
__device__ __forceinline__ double block_sum(double v, double* sh) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = (lane < NT / 32) ? sh[lane] : 0.0;
        r = warp_sum(r);
    }
    return r;
}

int grid_for(int64_t n, int cap) {
    int64_t g = (n + NT * 4 - 1) / (NT * 4);
    g = (g + NSM - 1) / NSM * NSM;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

__global__ void __launch_bounds__(NT) dot_partial(const double* __restrict__ x,
                                                  const double* __restrict__ y, int64_t n,
                                                  double* __restrict__ red) {
    __shared__ double sh[NT / 32];
    double acc = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT)
        acc = fma(x[i], y ? y[i] : x[i], acc);
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) red[blockIdx.x] = acc;
}

__global__ void __launch_bounds__(NT) sum_partials(const double* __restrict__ red, int nb,
                                                   int stride, int nrow, int take_sqrt,
                                                   double* __restrict__ out) {
    __shared__ double sh[NT / 32];
    for (int row = 0; row < nrow; ++row) {
        double acc = 0.0;
        for (int b = threadIdx.x; b < nb; b += NT) acc += red[(int64_t)b * stride + row];
        acc = block_sum(acc, sh);
        if (threadIdx.x == 0) out[row] = take_sqrt ? sqrt(acc) : acc;
    }
}

// Partial c[i] over this CTA's chunk of k, MD_ROWS rows of V at a time (w is re-read from L1).
__global__ void __launch_bounds__(NT) multidot_partial(const double* __restrict__ V, int64_t ldv,
                                                       int nv, const double* __restrict__ w,
                                                       int64_t n, double* __restrict__ red) {
    __shared__ double sh[NT / 32];
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t k0 = blockIdx.x * chunk;
    const int64_t k1 = min(n, k0 + chunk);
    for (int i0 = 0; i0 < nv; i0 += MD_ROWS) {
        double acc[MD_ROWS];
#pragma unroll
        for (int r = 0; r < MD_ROWS; ++r) acc[r] = 0.0;
        for (int64_t k = k0 + threadIdx.x; k < k1; k += NT) {
            const double wk = w[k];
#pragma unroll
            for (int r = 0; r < MD_ROWS; ++r)
                if (i0 + r < nv) acc[r] = fma(V[(int64_t)(i0 + r) * ldv + k], wk, acc[r]);
        }
#pragma unroll
        for (int r = 0; r < MD_ROWS; ++r) {
            if (i0 + r >= nv) break;
            const double s = block_sum(acc[r], sh);
            if (threadIdx.x == 0) red[(int64_t)blockIdx.x * MAXNV + i0 + r] = s;
        }
    }
}

__global__ void __launch_bounds__(NT) gemv_sub_kernel(const double* __restrict__ V, int64_t ldv,
                                                      int nv, const double* __restrict__ c,
                                                      double* __restrict__ w, int64_t n) {
    __shared__ double cs[MAXNV];
    if (threadIdx.x < nv) cs[threadIdx.x] = c[threadIdx.x];
    __syncthreads();
    for (int64_t k = blockIdx.x * (int64_t)NT + threadIdx.x; k < n; k += (int64_t)gridDim.x * NT) {
        double acc = w[k];
        for (int i = 0; i < nv; ++i) acc = fma(-cs[i], V[(int64_t)i * ldv + k], acc);
        w[k] = acc;
    }
}

__global__ void __launch_bounds__(NT) axpby_kernel(const double* __restrict__ x,
                                                   double* __restrict__ y, int64_t n,
                                                   const double* sa, double fa, const double* sb,
                                                   double fb) {
    const double a = (sa ? sa[0] : 1.0) * fa;
    const double b = (sb ? sb[0] : 1.0) * fb;
    for (int64_t k = blockIdx.x * (int64_t)NT + threadIdx.x; k < n; k += (int64_t)gridDim.x * NT)
        y[k] = (b == 0.0) ? a * x[k] : fma(a, x[k], b * y[k]);
}

__global__ void __launch_bounds__(NT) scale_div_kernel(const double* __restrict__ x,
                                                       double* __restrict__ y, int64_t n,
                                                       const double* s, double f) {
    const double a = f / s[0];
    for (int64_t k = blockIdx.x * (int64_t)NT + threadIdx.x; k < n; k += (int64_t)gridDim.x * NT)
        y[k] = x[k] * a;
}

}  // namespace

int vec_dot(const double* x, const double* y, int64_t n, double* out, double* red,
            int take_sqrt, cudaStream_t stream) {
    if (!x || !out || !red || n < 0) {
        set_error("dot/nrm2: bad argument");
        return TNK_ERR_ARG;
    }
    const int g = grid_for(n, 8 * NSM);
    dot_partial<<<g, NT, 0, stream>>>(x, y, n, red);
    int rc = check_launch("dot_partial");
    if (rc) return rc;
    sum_partials<<<1, NT, 0, stream>>>(red, g, 1, 1, take_sqrt, out);
    return check_launch("sum_partials");
}

int vec_multidot(const double* V, int64_t ldv, int nv, const double* w, int64_t n, double* c,
                 double* red, cudaStream_t stream) {
    if (!V || !w || !c || !red || n < 0 || nv < 0 || nv > MAXNV || ldv < n) {
        set_error("multidot: bad argument (nv=%d, n=%lld, ldv=%lld)", nv, (long long)n,
                  (long long)ldv);
        return TNK_ERR_ARG;
    }
    if (nv == 0) return TNK_OK;
    // partials: grid * MAXNV doubles must fit TNK_RED_ELEMS
    const int g = grid_for(n, TNK_RED_ELEMS / MAXNV);
    multidot_partial<<<g, NT, 0, stream>>>(V, ldv, nv, w, n, red);
    int rc = check_launch("multidot_partial");
    if (rc) return rc;
    sum_partials<<<1, NT, 0, stream>>>(red, g, MAXNV, nv, 0, c);
    return check_launch("sum_partials");
}

int vec_gemv_sub(const double* V, int64_t ldv, int nv, const double* c, double* w, int64_t n,
                 cudaStream_t stream) {
    if (!V || !w || !c || n < 0 || nv < 0 || nv > MAXNV || ldv < n) {
        set_error("gemv_sub: bad argument");
        return TNK_ERR_ARG;
    }
    if (nv == 0 || n == 0) return TNK_OK;
    gemv_sub_kernel<<<grid_for(n, 16 * NSM), NT, 0, stream>>>(V, ldv, nv, c, w, n);
    return check_launch("gemv_sub_kernel");
}

int vec_axpby(const double* x, double* y, int64_t n, const double* sa, double fa,
              const double* sb, double fb, cudaStream_t stream) {
    if (!x || !y || n < 0) {
        set_error("axpby: bad argument");
        return TNK_ERR_ARG;
    }
    if (n == 0) return TNK_OK;
    axpby_kernel<<<grid_for(n, 16 * NSM), NT, 0, stream>>>(x, y, n, sa, fa, sb, fb);
    return check_launch("axpby_kernel");
}

int vec_scale_div(const double* x, double* y, int64_t n, const double* s, double f,
                  cudaStream_t stream) {
    if (!x || !y || !s || n < 0) {
        set_error("scale_div: bad argument");
        return TNK_ERR_ARG;
    }
    if (n == 0) return TNK_OK;
    scale_div_kernel<<<grid_for(n, 16 * NSM), NT, 0, stream>>>(x, y, n, s, f);
    return check_launch("scale_div_kernel");
}

}  // namespace tnk
