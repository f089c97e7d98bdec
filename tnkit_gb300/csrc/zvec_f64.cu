// Complex128 Lanczos vector kernels (sm_103a) for the Krylov exponential of TDVP: vectors are
// interleaved (re, im) doubles. dot products conjugate their first argument, as numpy's vdot
// and the reference's `vdot` do; scalars are read from device memory so no call synchronises.
// Reductions are two-phase and deterministic, as in vec_f64.cu.
#include "tnk_internal.cuh"

namespace tnk {
namespace {

constexpr int NT = 256;
constexpr int NSM = 152;
constexpr int MAXNV = 64;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

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

int zgrid(int64_t n, int cap) {
    int64_t g = (n + NT * 2 - 1) / (NT * 2);
    g = (g + NSM - 1) / NSM * NSM;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

// partial sums of conj(x) y: red[2*b] (re), red[2*b+1] (im)
__global__ void __launch_bounds__(NT) zdot_partial(const double2* __restrict__ x,
                                                   const double2* __restrict__ y, int64_t n,
                                                   double* __restrict__ red) {
    __shared__ double sh[NT / 32];
    double re = 0.0, im = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT) {
        const double2 a = x[i], b = y[i];
        re = fma(a.x, b.x, fma(a.y, b.y, re));
        im = fma(a.x, b.y, fma(-a.y, b.x, im));
    }
    re = block_sum(re, sh);
    im = block_sum(im, sh);
    if (threadIdx.x == 0) {
        red[2 * blockIdx.x] = re;
        red[2 * blockIdx.x + 1] = im;
    }
}

// out[2*row + {0,1}] = sum over nb partials at red[b*stride + 2*row + {0,1}]
__global__ void __launch_bounds__(NT) zsum_partials(const double* __restrict__ red, int nb,
                                                    int stride, int nrow,
                                                    double* __restrict__ out) {
    __shared__ double sh[NT / 32];
    for (int row = 0; row < 2 * nrow; ++row) {
        double acc = 0.0;
        for (int b = threadIdx.x; b < nb; b += NT) acc += red[(int64_t)b * stride + row];
        acc = block_sum(acc, sh);
        if (threadIdx.x == 0) out[row] = acc;
    }
}

// c_i = sum_k conj(V[i, k]) w[k] for i < nv, partials per CTA chunk
__global__ void __launch_bounds__(NT) zmultidot_partial(const double2* __restrict__ V,
                                                        int64_t ldv, int nv,
                                                        const double2* __restrict__ w,
                                                        int64_t n, double* __restrict__ red) {
    __shared__ double sh[NT / 32];
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t k0 = blockIdx.x * chunk;
    const int64_t k1 = min(n, k0 + chunk);
    for (int i = 0; i < nv; ++i) {
        double re = 0.0, im = 0.0;
        for (int64_t k = k0 + threadIdx.x; k < k1; k += NT) {
            const double2 a = V[(int64_t)i * ldv + k], b = w[k];
            re = fma(a.x, b.x, fma(a.y, b.y, re));
            im = fma(a.x, b.y, fma(-a.y, b.x, im));
        }
        re = block_sum(re, sh);
        im = block_sum(im, sh);
        if (threadIdx.x == 0) {
            red[(int64_t)blockIdx.x * 2 * MAXNV + 2 * i] = re;
            red[(int64_t)blockIdx.x * 2 * MAXNV + 2 * i + 1] = im;
        }
    }
}

// w[k] -= sum_i c_i V[i, k] (complex c from device memory)
__global__ void __launch_bounds__(NT) zgemv_sub_kernel(const double2* __restrict__ V,
                                                       int64_t ldv, int nv,
                                                       const double2* __restrict__ c,
                                                       double2* __restrict__ w, int64_t n) {
    __shared__ double2 cs[MAXNV];
    if (threadIdx.x < nv) cs[threadIdx.x] = c[threadIdx.x];
    __syncthreads();
    for (int64_t k = blockIdx.x * (int64_t)NT + threadIdx.x; k < n; k += (int64_t)gridDim.x * NT) {
        double2 acc = w[k];
        for (int i = 0; i < nv; ++i) {
            const double2 v = V[(int64_t)i * ldv + k], a = cs[i];
            acc.x -= a.x * v.x - a.y * v.y;
            acc.y -= a.x * v.y + a.y * v.x;
        }
        w[k] = acc;
    }
}

// y = a x + b y, a = (sa ? sa : 1) * fa, b = (sb ? sb : 1) * fb, sa/sb complex on the device
__global__ void __launch_bounds__(NT) zaxpby_kernel(const double2* __restrict__ x,
                                                    double2* __restrict__ y, int64_t n,
                                                    const double2* sa, double fa,
                                                    const double2* sb, double fb) {
    const double2 a0 = sa ? sa[0] : make_double2(1.0, 0.0);
    const double2 b0 = sb ? sb[0] : make_double2(1.0, 0.0);
    const double ar = a0.x * fa, ai = a0.y * fa, br = b0.x * fb, bi = b0.y * fb;
    const bool keep_y = (br != 0.0 || bi != 0.0);
    for (int64_t k = blockIdx.x * (int64_t)NT + threadIdx.x; k < n; k += (int64_t)gridDim.x * NT) {
        const double2 u = x[k];
        double2 r = make_double2(ar * u.x - ai * u.y, ar * u.y + ai * u.x);
        if (keep_y) {
            const double2 v = y[k];
            r.x += br * v.x - bi * v.y;
            r.y += br * v.y + bi * v.x;
        }
        y[k] = r;
    }
}

}  // namespace

int zvec_dot(const double* x, const double* y, int64_t n, double* out, double* red,
             cudaStream_t st) {
    if (!x || !y || !out || !red || n < 0) {
        set_error("zdot: bad argument");
        return TNK_ERR_ARG;
    }
    const int g = zgrid(n, TNK_RED_ELEMS / 2 < 8 * NSM ? TNK_RED_ELEMS / 2 : 8 * NSM);
    zdot_partial<<<g, NT, 0, st>>>(reinterpret_cast<const double2*>(x),
                                   reinterpret_cast<const double2*>(y), n, red);
    int rc = check_launch("zdot_partial");
    if (rc) return rc;
    zsum_partials<<<1, NT, 0, st>>>(red, g, 2, 1, out);
    return check_launch("zsum_partials");
}

int zvec_multidot(const double* V, int64_t ldv, int nv, const double* w, int64_t n, double* c,
                  double* red, cudaStream_t st) {
    if (!V || !w || !c || !red || n < 0 || nv < 0 || nv > MAXNV || ldv < n) {
        set_error("zmultidot: bad argument");
        return TNK_ERR_ARG;
    }
    if (nv == 0) return TNK_OK;
    const int g = zgrid(n, TNK_RED_ELEMS / (2 * MAXNV));
    zmultidot_partial<<<g, NT, 0, st>>>(reinterpret_cast<const double2*>(V), ldv, nv,
                                        reinterpret_cast<const double2*>(w), n, red);
    int rc = check_launch("zmultidot_partial");
    if (rc) return rc;
    zsum_partials<<<1, NT, 0, st>>>(red, g, 2 * MAXNV, nv, c);
    return check_launch("zsum_partials");
}

int zvec_gemv_sub(const double* V, int64_t ldv, int nv, const double* c, double* w, int64_t n,
                  cudaStream_t st) {
    if (!V || !w || !c || n < 0 || nv < 0 || nv > MAXNV || ldv < n) {
        set_error("zgemv_sub: bad argument");
        return TNK_ERR_ARG;
    }
    if (nv == 0 || n == 0) return TNK_OK;
    zgemv_sub_kernel<<<zgrid(n, 16 * NSM), NT, 0, st>>>(
        reinterpret_cast<const double2*>(V), ldv, nv, reinterpret_cast<const double2*>(c),
        reinterpret_cast<double2*>(w), n);
    return check_launch("zgemv_sub_kernel");
}

int zvec_axpby(const double* x, double* y, int64_t n, const double* sa, double fa,
               const double* sb, double fb, cudaStream_t st) {
    if (!x || !y || n < 0) {
        set_error("zaxpby: bad argument");
        return TNK_ERR_ARG;
    }
    if (n == 0) return TNK_OK;
    zaxpby_kernel<<<zgrid(n, 16 * NSM), NT, 0, st>>>(
        reinterpret_cast<const double2*>(x), reinterpret_cast<double2*>(y), n,
        reinterpret_cast<const double2*>(sa), fa, reinterpret_cast<const double2*>(sb), fb);
    return check_launch("zaxpby_kernel");
}

}  // namespace tnk

extern "C" {

int tnk_zdot_f64(const double* x, const double* y, int64_t n, double* out, double* red,
                 void* stream) {
    return tnk::zvec_dot(x, y, n, out, red, (cudaStream_t)stream);
}

int tnk_zmultidot_f64(const double* V, int64_t ldv, int32_t nv, const double* w, int64_t n,
                      double* c, double* red, void* stream) {
    return tnk::zvec_multidot(V, ldv, nv, w, n, c, red, (cudaStream_t)stream);
}

int tnk_zgemv_sub_f64(const double* V, int64_t ldv, int32_t nv, const double* c, double* w,
                      int64_t n, void* stream) {
    return tnk::zvec_gemv_sub(V, ldv, nv, c, w, n, (cudaStream_t)stream);
}

int tnk_zaxpby_f64(const double* x, double* y, int64_t n, const double* sa, double fa,
                   const double* sb, double fb, void* stream) {
    return tnk::zvec_axpby(x, y, n, sa, fa, sb, fb, (cudaStream_t)stream);
}

}  // extern "C"
