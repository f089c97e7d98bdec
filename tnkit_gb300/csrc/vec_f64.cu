// Lanczos vector kernels (FP64, sm_103a): dot, norm, the passes of classical Gram-Schmidt
// (fused subtract / multi-dot / norm over one read of the basis), and scalar updates that read
// their scalars from device memory.
//
// All are HBM-bound streams. Reductions are deterministic: each CTA writes its partials
// (warp-shuffle, then shared-memory reduction), and one CTA sums them in a fixed order -- the
// last CTA of the same launch when the caller passes a counter, else a second launch. Grids are
// the resident CTAs of all SMs (or multiples of the 152 SMs), capped so the partials fit the
// caller's TNK_RED_ELEMS workspace.
#include <atomic>

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

// Transposed warp reduction of G (16 or 32) values per lane: on return, lane l holds the sum
// over the warp's lanes of their v[l % G] (G = 16: both half-warps added at the end). Each step
// sends the half of the values a lane does not keep to its partner and adds the half it
// receives: G - 1 shuffle-adds instead of 5 per value, in a fixed order (deterministic).
template <int G>
__device__ __forceinline__ double warp_transpose_sum(double (&v)[G]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int s = G / 2; s >= 1; s >>= 1) {
        const bool up = (lane & s) != 0;
#pragma unroll
        for (int i = 0; i < s; ++i) {
            const double keep = up ? v[i + s] : v[i];
            const double send = up ? v[i] : v[i + s];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, s);
        }
    }
    if (G == 16) v[0] += __shfl_xor_sync(0xffffffffu, v[0], 16);
    return v[0];
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

// ---- fused classical Gram-Schmidt pass -------------------------------------------------------
// One read of the basis rows V[0..nv) serves up to two steps of CGS2 (mode bits):
//   CG_SUB  w[k] -= sum_i cin[i] V[i,k]
//   CG_DOT  c[i] = sum_k V[i,k] w[k]             (w after the subtraction)
//   CG_NRM  s = sqrt(sum_k w[k]^2)               (w after the subtraction)
// On GB300 these passes are bound by the FP64 pipe (~0.9 TFLOP/s for scalar FP64), not by HBM,
// so the kernel spends one FP64 FMA per element and row and little else: one thread per
// column, the subtraction as two interleaved FMA chains (even and odd rows, joined by one add)
// to halve its dependent latency, and shared-memory tiles small enough for several CTAs per SM,
// whose warps hide the FP64 latency. The k range is cut into tiles of CG_TK columns that stream
// through a ring of 2..8 stages in shared memory, filled with asynchronous 8-byte copies
// (cp.async, zero fill past n); each thread copies and reads only its own column, so the ring
// needs no barrier. Each CTA writes its partials to red[cta * PSTRIDE + row]. The sum over CTAs
// runs in one CTA, in a fixed order: the partials are copied into shared memory in one batch
// (16-byte cp.async.cg, so L2 and not a stale L1 line is read) and summed per row. With a
// counter, that CTA is the last of the launch to finish (atomic ticket after a fence), which
// also resets the counter; without one, finish_kernel is a second launch.
constexpr int CG_SUB = 1, CG_DOT = 2, CG_NRM = 4;
constexpr int PSTRIDE = MAXNV + 2;     // even: every CTA's partial row starts 16-byte aligned
constexpr int CG_TK = 128;             // columns per tile = threads per CTA
constexpr int CG_NT = CG_TK;
constexpr int CG_RING_BYTES = 48 * 1024;
constexpr int CG_MAX_STAGES = 8;

// ring stages and bytes for nv rows of `es`-byte elements
__host__ __device__ inline int cg_stages(int nv, int es) {
    int s = CG_RING_BYTES / ((nv + 1) * CG_TK * es);
    return s < 2 ? 2 : (s > CG_MAX_STAGES ? CG_MAX_STAGES : s);
}

__host__ __device__ inline int cg_ring_bytes(int nv, int es) {
    return cg_stages(nv, es) * (nv + 1) * CG_TK * es;
}

// partial rows of one CTA, rounded up to an even count (16-byte copies)
__host__ __device__ inline int cg_prow(int mode, int nv) {
    const int r = (mode & CG_DOT) && nv > 1 ? nv : 1;
    return (r + 1) & ~1;
}

__device__ __forceinline__ void cp_async_elem(double* dst, const double* src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src),
                 "r"(valid ? 8 : 0)
                 : "memory");
}

__device__ __forceinline__ void cp_async_elem(float* dst, const float* src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src),
                 "r"(valid ? 4 : 0)
                 : "memory");
}

__device__ __forceinline__ void cp_async16_cg(double* dst, const double* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// wait until at most `pending` (0..CG_MAX_STAGES-1) of this thread's copy groups are in flight
__device__ __forceinline__ void cp_async_wait_dyn(int pending) {
    switch (pending) {
        case 0: asm volatile("cp.async.wait_group 0;\n" ::: "memory"); break;
        case 1: asm volatile("cp.async.wait_group 1;\n" ::: "memory"); break;
        case 2: asm volatile("cp.async.wait_group 2;\n" ::: "memory"); break;
        case 3: asm volatile("cp.async.wait_group 3;\n" ::: "memory"); break;
        case 4: asm volatile("cp.async.wait_group 4;\n" ::: "memory"); break;
        case 5: asm volatile("cp.async.wait_group 5;\n" ::: "memory"); break;
        case 6: asm volatile("cp.async.wait_group 6;\n" ::: "memory"); break;
        default: asm volatile("cp.async.wait_group 7;\n" ::: "memory"); break;
    }
}

// Sum the partials of `nb` CTAs (prow doubles each, the first `nrow` used) into out[0..nrow),
// square-rooted when `root`. Runs in one whole CTA of CG_NT threads. The partials pass through
// `stage` (stage_elems doubles) in chunks of CTAs, each chunk copied in one batch; each row is
// split among CG_NT / nrow threads (strided CTA subsets, summed in increasing CTA order), whose
// sums are then added in a fixed order: the result does not depend on timing.
__device__ void finish_partials(const double* red, int nb, int prow, int nrow, bool root,
                                double* stage, int stage_elems, double* out) {
    __shared__ double part[CG_NT];
    const int half = prow / 2;
    const int G = nrow > 0 ? CG_NT / nrow : 1;       // threads per row (nrow <= 64)
    const int idx = threadIdx.x;
    const int r = idx / G, g = idx - r * G;
    const bool active = idx < nrow * G;
    const int cap = stage_elems / prow > 0 ? stage_elems / prow : 1;
    double s = 0.0;
    for (int b0 = 0; b0 < nb; b0 += cap) {
        const int b1 = nb - b0 < cap ? nb : b0 + cap;
        __syncthreads();                              // the previous chunk has been read
        for (int e = idx; e < (b1 - b0) * half; e += blockDim.x) {
            const int b = e / half, h = e - b * half;
            cp_async16_cg(stage + (int64_t)b * prow + 2 * h,
                          red + (int64_t)(b0 + b) * PSTRIDE + 2 * h);
        }
        cp_async_commit();
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        __syncthreads();
        if (active) {
            int b = b0 + ((g - b0 % G) % G + G) % G;  // first b >= b0 with b = g (mod G)
            for (; b < b1; b += G) s += stage[(int64_t)(b - b0) * prow + r];
        }
    }
    if (active) part[idx] = s;
    __syncthreads();
    if (idx < nrow) {
        double t = 0.0;
        for (int q = 0; q < G; ++q) t += part[idx * G + q];
        out[idx] = root ? sqrt(t) : t;
    }
}

constexpr int CG_FIN_ELEMS = 4096;                   // staging of finish_kernel (32 KB)

__global__ void __launch_bounds__(CG_NT) finish_kernel(const double* __restrict__ red, int nb,
                                                      int prow, int nrow, int root,
                                                      double* __restrict__ out) {
    __shared__ __align__(16) double fin[CG_FIN_ELEMS];
    finish_partials(red, nb, prow, nrow, root != 0, fin, CG_FIN_ELEMS, out);
}

// Segmented launches: many independent vectors (chains) concatenated in one batch vector, chain
// c at [off[c], off[c+1]); grid row y works on chain ids[y] alone, with its own coefficient
// vector cin + c*rec_stride, output out + c*rec_stride, partial rows and completion counter
// (counter + y): one launch performs the pass of every listed chain, no reduction mixing them.
struct CgsSeg {
    const int64_t* off;          // null: one segment, the plain pass
    const int32_t* ids;
    int64_t rec_stride;
};

template <typename T, int NVB, int MODE>
__global__ void __launch_bounds__(CG_NT) cgs_kernel(const T* __restrict__ V, int64_t ldv, int nv,
                                                   const double* __restrict__ cin,
                                                   T* __restrict__ w, int64_t n,
                                                   double* __restrict__ red,
                                                   unsigned* __restrict__ counter,
                                                   double* __restrict__ out, CgsSeg seg) {
    if (seg.off) {
        const int c = seg.ids[blockIdx.y];
        const int64_t a = seg.off[c];
        n = seg.off[c + 1] - a;
        V += a;
        w += a;
        if (cin) cin += (int64_t)c * seg.rec_stride;
        if (out) out += (int64_t)c * seg.rec_stride;
        if (red) red += (int64_t)blockIdx.y * gridDim.x * PSTRIDE;
        if (counter) counter += blockIdx.y;
    }
    constexpr bool SUB = (MODE & CG_SUB) != 0;
    constexpr bool DOT = (MODE & CG_DOT) != 0;
    constexpr bool NRM = (MODE & CG_NRM) != 0;
    constexpr int NACC = DOT ? NVB : 1;
    extern __shared__ __align__(16) unsigned char ring_raw[];
    T* ring = reinterpret_cast<T*>(ring_raw);        // [stage][row 0: w, rows 1..nv: V][CG_TK]
    __shared__ T cs[NVB];
    __shared__ double sh[CG_NT / 32][NVB + 1];
    __shared__ bool last;
    const int t = threadIdx.x;
    const int rows = nv + 1;
    const int stages = cg_stages(nv, (int)sizeof(T));
    if (SUB && t < NVB) cs[t] = t < nv ? (T)(-cin[t]) : (T)0;
    __syncthreads();
    const int64_t ntiles = (n + CG_TK - 1) / CG_TK;

    auto issue = [&](int64_t tile, int slot) {
        if (tile < ntiles) {
            const int64_t k = tile * CG_TK + t;
            const bool ok = k < n;
            const int64_t kk = ok ? k : 0;
            T* st = ring + (int64_t)slot * rows * CG_TK + t;
            cp_async_elem(st, w + kk, ok);
            for (int i = 0; i < nv; ++i)
                cp_async_elem(st + (i + 1) * CG_TK, V + (int64_t)i * ldv + kk, ok);
        }
        cp_async_commit();
    };

    T acc[NACC];
#pragma unroll
    for (int i = 0; i < NACC; ++i) acc[i] = (T)0;
    T accn = (T)0;
    int64_t tile = blockIdx.x;
    for (int s = 0; s < stages - 1; ++s) issue(tile + (int64_t)s * gridDim.x, s);
    int slot = 0;
    for (; tile < ntiles; tile += gridDim.x) {
        cp_async_wait_dyn(stages - 2);
        issue(tile + (int64_t)(stages - 1) * gridDim.x, slot == 0 ? stages - 1 : slot - 1);
        const T* st = ring + (int64_t)slot * rows * CG_TK + t;
        const int64_t k = tile * CG_TK + t;
        T wk = st[0];
        if (SUB) {
            T s1 = (T)0;
            int i = 0;
            for (; i + 1 < nv; i += 2) {
                wk = fma(cs[i], st[(i + 1) * CG_TK], wk);
                s1 = fma(cs[i + 1], st[(i + 2) * CG_TK], s1);
            }
            if (i < nv) wk = fma(cs[i], st[(i + 1) * CG_TK], wk);
            wk += s1;
            if (k < n) w[k] = wk;
        }
        if (DOT) {
#pragma unroll
            for (int j = 0; j < NACC; ++j)
                if (j < nv) acc[j] = fma(st[(j + 1) * CG_TK], wk, acc[j]);
        }
        if (NRM) accn = fma(wk, wk, accn);
        slot = slot + 1 == stages ? 0 : slot + 1;
    }
    cp_async_wait_dyn(0);
    if (!DOT && !NRM) return;
    const int lane = t & 31, wid = t >> 5;
    if (DOT) {
        constexpr int G = NACC < 32 ? NACC : 32;
#pragma unroll
        for (int g = 0; g < NACC / G; ++g) {
            double v[G];
#pragma unroll
            for (int i = 0; i < G; ++i) v[i] = (double)acc[g * G + i];
            const double s = warp_transpose_sum<G>(v);
            const int row = g * G + (lane % G);
            if (lane < G && row < nv) sh[wid][row] = s;
        }
    }
    if (NRM) {
        const double s = warp_sum((double)accn);
        if (lane == 0) sh[wid][0] = s;
    }
    __syncthreads();
    const int nrow = DOT ? nv : 1;
    double* part = red + (int64_t)blockIdx.x * PSTRIDE;
    if (t < nrow) {
        double s = 0.0;
        for (int y = 0; y < CG_NT / 32; ++y) s += sh[y][t];
        part[t] = s;
    }
    if (!counter) return;
    __threadfence();
    __syncthreads();
    if (t == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    // the ring is idle now: it stages the partials
    finish_partials(red, gridDim.x, cg_prow(MODE, nv), nrow, NRM,
                    reinterpret_cast<double*>(ring_raw),
                    stages * rows * CG_TK * (int)sizeof(T) / (int)sizeof(double), out);
    if (t == 0) *counter = 0u;
}

// Grid size: one CTA per tile, at most the resident CTAs of all SMs and TNK_RED_ELEMS / PSTRIDE.
template <typename T, int NVB, int MODE>
int cgs_grid(int64_t n, int nv) {
    constexpr int ES = (int)sizeof(T);
    // per device: the opt-in to the largest ring; per row count: the resident CTAs per SM
    static std::atomic<unsigned long long> opted{0};
    static std::atomic<int> nsm{0};
    static std::atomic<int> occ_of[MAXNV + 1];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(opted.load(std::memory_order_acquire) & bit)) {
        int big = 0;
        for (int v = 0; v <= NVB; ++v)
            big = cg_ring_bytes(v, ES) > big ? cg_ring_bytes(v, ES) : big;
        cudaFuncSetAttribute(cgs_kernel<T, NVB, MODE>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, big);
        int cnt = 0;
        if (cudaDeviceGetAttribute(&cnt, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cnt < 1)
            cnt = NSM;
        nsm.store(cnt, std::memory_order_relaxed);
        opted.fetch_or(bit, std::memory_order_acq_rel);
    }
    int occ = occ_of[nv].load(std::memory_order_relaxed);
    if (occ < 1) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, cgs_kernel<T, NVB, MODE>, CG_NT,
                                                          cg_ring_bytes(nv, ES)) !=
                cudaSuccess ||
            occ < 1)
            occ = 1;
        occ_of[nv].store(occ, std::memory_order_relaxed);
    }
    int64_t cap = (int64_t)occ * nsm.load(std::memory_order_relaxed);
    if (cap > TNK_RED_ELEMS / PSTRIDE) cap = TNK_RED_ELEMS / PSTRIDE;
    int64_t g = (n + CG_TK - 1) / CG_TK;
    if (g > cap) g = cap;
    return g < 1 ? 1 : (int)g;
}

template <typename T, int NVB, int MODE>
int launch_cgs_t(const T* V, int64_t ldv, int nv, const double* cin, T* w, int64_t n,
                 double* red, unsigned* counter, double* out, cudaStream_t st,
                 CgsSeg seg = CgsSeg{nullptr, nullptr, 0}, int nseg = 1) {
    int g = cgs_grid<T, NVB, MODE>(n, nv);
    if (seg.off) {
        // every chain gets the same number of CTAs; all of their partial rows fit the
        // reduction buffer (n here is the longest segment)
        const int per = (TNK_RED_ELEMS / PSTRIDE) / nseg;
        g = g > per ? per : g;
        g = g < 1 ? 1 : g;
        cgs_kernel<T, NVB, MODE><<<dim3(g, nseg), CG_NT, cg_ring_bytes(nv, (int)sizeof(T)), st>>>(
            V, ldv, nv, cin, w, n, red, counter, out, seg);
        return check_launch("cgs_kernel (segmented)");
    }
    cgs_kernel<T, NVB, MODE><<<g, CG_NT, cg_ring_bytes(nv, (int)sizeof(T)), st>>>(
        V, ldv, nv, cin, w, n, red, counter, out, seg);
    int rc = check_launch("cgs_kernel");
    if (rc || counter || !(MODE & (CG_DOT | CG_NRM))) return rc;
    finish_kernel<<<1, CG_NT, 0, st>>>(red, g, cg_prow(MODE, nv), (MODE & CG_DOT) ? nv : 1,
                                       (MODE & CG_NRM) ? 1 : 0, out);
    return check_launch("finish_kernel");
}

// One launch of a fixed mode over nv <= 64 rows (NVB, the accumulator count, picked from nv).
template <int MODE, typename T>
int launch_cgs(const T* V, int64_t ldv, int nv, const double* cin, T* w, int64_t n,
               double* red, unsigned* counter, double* out, cudaStream_t st,
               CgsSeg seg = CgsSeg{nullptr, nullptr, 0}, int nseg = 1) {
    if (nv <= 16)
        return launch_cgs_t<T, 16, MODE>(V, ldv, nv, cin, w, n, red, counter, out, st, seg, nseg);
    if (nv <= 32)
        return launch_cgs_t<T, 32, MODE>(V, ldv, nv, cin, w, n, red, counter, out, st, seg, nseg);
    return launch_cgs_t<T, 64, MODE>(V, ldv, nv, cin, w, n, red, counter, out, st, seg, nseg);
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

__global__ void __launch_bounds__(NT) scale_div_f32_kernel(const float* __restrict__ x,
                                                           float* __restrict__ y, int64_t n,
                                                           const double* s, double f) {
    const float a = (float)(f / s[0]);
    for (int64_t k = blockIdx.x * (int64_t)NT + threadIdx.x; k < n; k += (int64_t)gridDim.x * NT)
        y[k] = x[k] * a;
}

__global__ void __launch_bounds__(NT) scale_div_kernel(const double* __restrict__ x,
                                                       double* __restrict__ y, int64_t n,
                                                       const double* s, double f) {
    const double a = f / s[0];
    for (int64_t k = blockIdx.x * (int64_t)NT + threadIdx.x; k < n; k += (int64_t)gridDim.x * NT)
        y[k] = x[k] * a;
}

// Segmented scale: grid row y scales chain ids[y]'s segment [off[c], off[c+1]) of x into y by
// f / s[c * s_stride] (each chain its own device scalar).
__global__ void __launch_bounds__(NT) scale_div_seg_kernel(const double* __restrict__ x,
                                                           double* __restrict__ y,
                                                           const int64_t* __restrict__ off,
                                                           const int32_t* __restrict__ ids,
                                                           const double* s, int64_t s_stride,
                                                           double f) {
    const int c = ids[blockIdx.y];
    const int64_t a = off[c], n = off[c + 1] - a;
    const double m = f / s[(int64_t)c * s_stride];
    for (int64_t k = blockIdx.x * (int64_t)NT + threadIdx.x; k < n; k += (int64_t)gridDim.x * NT)
        y[a + k] = x[a + k] * m;
}

// Thick-restart rotation of an FP32 Krylov basis: out[q*ldo + k] = sum_r Y[r*kk + q] V[r*ldv + k]
// (q < kk kept Ritz vectors, r < nv basis rows, r ascending). One thread per column k: the
// coefficients, converted to FP32 and padded with zeros to a multiple of RQ columns, sit in
// shared memory and are read as broadcast float4; V is read once per chunk of RQ outputs (once
// for kk <= RQ), coalesced along k.
constexpr int RQ = 16;

__global__ void __launch_bounds__(NT) rotate_f32_kernel(const float* __restrict__ V, int64_t ldv,
                                                        int nv, const double* __restrict__ Y,
                                                        int kk, float* __restrict__ out,
                                                        int64_t ldo, int64_t n) {
    __shared__ __align__(16) float ys[MAXNV * MAXNV];
    const int kp = (kk + RQ - 1) / RQ * RQ;
    for (int i = threadIdx.x; i < nv * kp; i += NT) {
        const int r = i / kp, q = i - r * kp;
        ys[i] = q < kk ? (float)Y[r * kk + q] : 0.0f;
    }
    __syncthreads();
    for (int64_t k = blockIdx.x * (int64_t)NT + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * NT) {
        for (int q0 = 0; q0 < kk; q0 += RQ) {
            float acc[RQ];
#pragma unroll
            for (int q = 0; q < RQ; ++q) acc[q] = 0.0f;
#pragma unroll 4
            for (int r = 0; r < nv; ++r) {
                const float v = V[r * ldv + k];
                const float4* y4 = reinterpret_cast<const float4*>(ys + r * kp + q0);
#pragma unroll
                for (int c = 0; c < RQ / 4; ++c) {
                    const float4 y = y4[c];
                    acc[4 * c + 0] = fmaf(y.x, v, acc[4 * c + 0]);
                    acc[4 * c + 1] = fmaf(y.y, v, acc[4 * c + 1]);
                    acc[4 * c + 2] = fmaf(y.z, v, acc[4 * c + 2]);
                    acc[4 * c + 3] = fmaf(y.w, v, acc[4 * c + 3]);
                }
            }
#pragma unroll
            for (int q = 0; q < RQ; ++q)
                if (q0 + q < kk) out[(q0 + q) * ldo + k] = acc[q];
        }
    }
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
    if (!V || !w || !c || !red || ((uintptr_t)red & 15) || n < 0 || nv < 0 || nv > MAXNV ||
        ldv < n) {
        set_error("multidot: bad argument (nv=%d, n=%lld, ldv=%lld)", nv, (long long)n,
                  (long long)ldv);
        return TNK_ERR_ARG;
    }
    if (nv == 0) return TNK_OK;
    return launch_cgs<CG_DOT, double>(V, ldv, nv, nullptr, const_cast<double*>(w), n, red,
                                      nullptr, c, stream);
}

int vec_gemv_sub(const double* V, int64_t ldv, int nv, const double* c, double* w, int64_t n,
                 cudaStream_t stream) {
    if (!V || !w || !c || n < 0 || nv < 0 || nv > MAXNV || ldv < n) {
        set_error("gemv_sub: bad argument");
        return TNK_ERR_ARG;
    }
    if (nv == 0 || n == 0) return TNK_OK;
    return launch_cgs<CG_SUB>(V, ldv, nv, c, w, n, nullptr, nullptr, nullptr, stream);
}

template <typename T>
int cgs_pass_t(const T* V, int64_t ldv, int nv, const double* cin, T* w, int64_t n, double* out,
               int mode, double* red, unsigned* counter, cudaStream_t st) {
    const bool sub = mode & CG_SUB, dot = mode & CG_DOT, nrm = mode & CG_NRM;
    if (n < 0 || nv < 0 || nv > MAXNV || mode < 1 || mode > 7 || (dot && nrm) ||
        (n > 0 && !w) || ((sub || dot) && (ldv < n || (n > 0 && nv > 0 && !V))) ||
        (sub && !cin) ||
        ((dot || nrm) && (!out || !red || ((uintptr_t)red & 15) || !counter))) {
        set_error("cgs_pass: bad argument (mode=%d, nv=%d, n=%lld, ldv=%lld)", mode, nv,
                  (long long)n, (long long)ldv);
        return TNK_ERR_ARG;
    }
    switch (mode) {
        case CG_SUB:
            if (nv == 0) return TNK_OK;
            return launch_cgs<CG_SUB>(V, ldv, nv, cin, w, n, nullptr, nullptr, nullptr, st);
        case CG_DOT:
            return launch_cgs<CG_DOT>(V, ldv, nv, cin, w, n, red, counter, out, st);
        case CG_SUB | CG_DOT:
            return launch_cgs<CG_SUB | CG_DOT>(V, ldv, nv, cin, w, n, red, counter, out, st);
        case CG_NRM:
            return launch_cgs<CG_NRM>(V, ldv, 0, nullptr, w, n, red, counter, out, st);
        default:  // CG_SUB | CG_NRM
            return launch_cgs<CG_SUB | CG_NRM>(V, ldv, nv, cin, w, n, red, counter, out, st);
    }
}

int vec_cgs_pass(const double* V, int64_t ldv, int nv, const double* cin, double* w, int64_t n,
                 double* out, int mode, double* red, unsigned* counter, cudaStream_t st) {
    return cgs_pass_t<double>(V, ldv, nv, cin, w, n, out, mode, red, counter, st);
}

// The segmented pass: chains ids[0..nseg) of the batch (offsets `off`, device arrays), the
// longest of them `max_len` entries, coefficient and output records rec_stride doubles apart,
// one completion counter per listed chain (counter[0..nseg), zero before the call and left
// zero after it).
int vec_cgs_pass_seg(const double* V, int64_t ldv, int nv, const double* cin, double* w,
                     const int64_t* off, const int32_t* ids, int nseg, int64_t max_len,
                     int64_t rec_stride, double* out, int mode, double* red, unsigned* counter,
                     cudaStream_t st) {
    const bool sub = mode & CG_SUB, dot = mode & CG_DOT, nrm = mode & CG_NRM;
    if (nseg < 0 || nseg > 65535 || max_len < 0 || nv < 0 || nv > MAXNV || mode < 1 ||
        mode > 7 || (dot && nrm) || (nseg > 0 && (!off || !ids || !w)) ||
        ((sub || dot) && (ldv < max_len || (nv > 0 && !V))) || (sub && !cin) ||
        ((dot || nrm) && (!out || !red || ((uintptr_t)red & 15) || !counter)) ||
        rec_stride < 0 || (nseg > 0 && (int64_t)nseg * PSTRIDE > TNK_RED_ELEMS)) {
        set_error("cgs_pass_seg: bad argument (mode=%d, nv=%d, nseg=%d, max_len=%lld)", mode, nv,
                  nseg, (long long)max_len);
        return TNK_ERR_ARG;
    }
    if (nseg == 0 || max_len == 0) return TNK_OK;
    const CgsSeg seg{off, ids, rec_stride};
    switch (mode) {
        case CG_SUB:
            if (nv == 0) return TNK_OK;
            return launch_cgs<CG_SUB>(V, ldv, nv, cin, w, max_len, nullptr, nullptr, nullptr, st,
                                      seg, nseg);
        case CG_DOT:
            return launch_cgs<CG_DOT>(V, ldv, nv, cin, w, max_len, red, counter, out, st, seg,
                                      nseg);
        case CG_SUB | CG_DOT:
            return launch_cgs<CG_SUB | CG_DOT>(V, ldv, nv, cin, w, max_len, red, counter, out,
                                               st, seg, nseg);
        case CG_NRM:
            return launch_cgs<CG_NRM>(V, ldv, 0, nullptr, w, max_len, red, counter, out, st, seg,
                                      nseg);
        default:  // CG_SUB | CG_NRM
            return launch_cgs<CG_SUB | CG_NRM>(V, ldv, nv, cin, w, max_len, red, counter, out,
                                               st, seg, nseg);
    }
}

int vec_cgs_pass_f32(const float* V, int64_t ldv, int nv, const double* cin, float* w,
                     int64_t n, double* out, int mode, double* red, unsigned* counter,
                     cudaStream_t st) {
    return cgs_pass_t<float>(V, ldv, nv, cin, w, n, out, mode, red, counter, st);
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

int vec_scale_div_seg(const double* x, double* y, const int64_t* off, const int32_t* ids,
                      int nseg, int64_t max_len, const double* s, int64_t s_stride, double f,
                      cudaStream_t stream) {
    if (nseg < 0 || nseg > 65535 || max_len < 0 || s_stride < 0 ||
        (nseg > 0 && (!x || !y || !off || !ids || !s))) {
        set_error("scale_div_seg: bad argument");
        return TNK_ERR_ARG;
    }
    if (nseg == 0 || max_len == 0) return TNK_OK;
    int64_t gx = (max_len + NT - 1) / NT;
    const int64_t cap = (16 * NSM + nseg - 1) / nseg;
    if (gx > cap) gx = cap;
    if (gx < 1) gx = 1;
    scale_div_seg_kernel<<<dim3((unsigned)gx, (unsigned)nseg), NT, 0, stream>>>(
        x, y, off, ids, s, s_stride, f);
    return check_launch("scale_div_seg_kernel");
}

int vec_scale_div_f32(const float* x, float* y, int64_t n, const double* s, double f,
                      cudaStream_t stream) {
    if (!x || !y || !s || n < 0) {
        set_error("scale_div_f32: bad argument");
        return TNK_ERR_ARG;
    }
    if (n == 0) return TNK_OK;
    scale_div_f32_kernel<<<grid_for(n, 16 * NSM), NT, 0, stream>>>(x, y, n, s, f);
    return check_launch("scale_div_f32_kernel");
}

int vec_rotate_f32(const float* V, int64_t ldv, int nv, const double* Y, int kk, float* out,
                   int64_t ldo, int64_t n, cudaStream_t stream) {
    if (n < 0 || nv < 0 || nv > MAXNV || kk < 1 || kk > MAXNV || ldv < n || ldo < n || !out ||
        (nv > 0 && (!Y || (n > 0 && !V)))) {
        set_error("rotate_f32: bad argument (nv=%d, kk=%d, n=%lld, ldv=%lld, ldo=%lld)", nv, kk,
                  (long long)n, (long long)ldv, (long long)ldo);
        return TNK_ERR_ARG;
    }
    if (n == 0) return TNK_OK;
    rotate_f32_kernel<<<grid_for(n, 16 * NSM), NT, 0, stream>>>(V, ldv, nv, Y, kk, out, ldo, n);
    return check_launch("rotate_f32_kernel");
}

}  // namespace tnk
