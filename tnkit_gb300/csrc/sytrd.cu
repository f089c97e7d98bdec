// The O(n^3) parts of the truncation's Gram route on the device, for every charge sector of a
// bond in one launch each: the Householder reduction of each sector's Gram matrix G = M M^T (or
// M^T M) to a symmetric tridiagonal T = Q^T G Q, and, once the tridiagonal eigenvectors Z of
// the kept singular values are known, their back-transformation U = Q Z. Together with the
// tridiagonal eigenproblem between them (O(n^2) with deflation), this is the eigh of
// tnkit/blocks.py:1345-1377 (method='gram') that the truncation of tnkit/blocks.py:1380-1462
// runs per sector.
//
// Reduction (sytrd_cluster_kernel). One thread-block cluster per sector; the sector's matrix
// stays in the distributed shared memory of its CTAs for the whole reduction: CTA r of a
// cluster of CS holds the full columns j = r, r + CS, r + 2 CS, ... (cyclic, so the shrinking
// trailing matrix stays balanced). Step k (Golub and Van Loan, Matrix Computations, 4th ed.,
// section 8.3.1): the owner of column k has formed the reflector H_k = I - tau v v^T that zeroes
// column k below its subdiagonal; every CTA copies v from the owner's shared memory, computes
// p_j = tau A[:, j] . v for its own columns, the cluster sums p . v, every CTA gathers the whole
// p from its peers and forms w = p - (tau/2)(p . v) v, and updates its own columns
// A -= v w^T + w v^T. The owner of column k + 1 updates that column first and forms the next
// reflector while the others finish their updates (look-ahead), so the only serial part of a
// step is two cluster barriers and the gathers. The work is FP64 FMA-bound: ~n^3 FMAs per
// sector over CS SMs. Outputs: the diagonal d, the off-diagonal e and tau per sector, and each
// reflector's v (v[k+1] = 1 stored) in column k, rows k+1 .. n-1, of the sector's G.
//
// Back-transformation (ormtr_cols_kernel). Columns are independent: each CTA takes up to
// ORM_COLS columns of one sector's Z, keeps them in shared memory and applies H_{n-3}, ..., H_0
// to them in turn (one warp per column; the reflectors are read from G, L2-resident, into a
// double-buffered shared vector).
//
// Neither kernel waits on a flag: the only waits are the hardware cluster and CTA barriers,
// which every thread of every CTA of a cluster reaches the same number of times (the loop
// counts depend only on the sector's order).
#include <cooperative_groups.h>

#include "tnk_internal.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int SY_THREADS = 256;
constexpr int SY_WARPS = SY_THREADS / 32;
constexpr int ORM_COLS = 8;                 // columns per CTA of the back-transformation
constexpr int ORM_THREADS = ORM_COLS * 32;  // one warp per column

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Shared-memory layout of a sector of order n on a cluster of cs CTAs (the same offsets in every
// CTA of the cluster, so peers address each other's arrays by the local offset). Columns are
// stored with an odd stride (ld = n | 1 doubles): threads that read one row of several
// columns then hit distinct banks.
struct SyShared {
    double* A;      // ncm columns of ld (the CTA's own columns, cyclic)
    double* vb;     // n: the reflector this CTA formed (read by the peers)
    double* vl;     // n: the current reflector
    double* wl;     // n: the current w
    double* pown;   // ncm: p of the own columns (read by the peers)
    double* part;   // SY_THREADS: partial column dot products
    double* scal;   // 2: tau of the reflector in vb, this CTA's share of p . v
};

__host__ __device__ inline int64_t sy_ld(int64_t n) { return n | 1; }

__host__ __device__ inline int64_t sy_shared_doubles(int64_t n, int cs) {
    const int64_t ncm = (n + cs - 1) / cs;
    return ncm * sy_ld(n) + 3 * n + ncm + SY_THREADS + 2;
}

__device__ SyShared sy_layout(double* sh, int n, int ncm) {
    SyShared s;
    s.A = sh;
    s.vb = s.A + (size_t)ncm * sy_ld(n);
    s.vl = s.vb + n;
    s.wl = s.vl + n;
    s.pown = s.wl + n;
    s.part = s.pown + ncm;
    s.scal = s.part + SY_THREADS;
    return s;
}

// The reflector of column c, formed by one warp (lanes over rows) from col (rows 0 .. n-1,
// already updated through step c - 1): H = I - tau v v^T with H [alpha; x] = [beta; 0],
// v = [1; x / (alpha - beta)], beta = -sign(alpha) ||[alpha; x]||, tau = (beta - alpha) / beta
// (tau = 0, v = e_1 when x = 0). The scalars are computed by lane 0 alone and broadcast. Writes
// v to vb and to column c of the sector's G (rows c+1 .. n-1), tau to scal[0] and tau[c], d[c]
// and e[c] = beta. The entries of a Gram matrix of a unit-norm block are at most 1 in magnitude,
// so the sum of squares needs no scaling (it underflows only below 1e-154).
__device__ void householder_warp(const double* col, int c, int n, double* vb, double* gcol,
                                 double* d, double* e, double* tau, double* scal) {
    const int lane = threadIdx.x & 31;
    const double alpha = col[c + 1];
    double ss = 0.0;
    for (int i = c + 2 + lane; i < n; i += 32) ss = fma(col[i], col[i], ss);
    ss = warp_sum(ss);
    double beta = alpha, t = 0.0, sc = 0.0;
    if (lane == 0 && ss > 0.0) {
        beta = -copysign(sqrt(fma(alpha, alpha, ss)), alpha);
        t = (beta - alpha) / beta;
        sc = 1.0 / (alpha - beta);
    }
    beta = __shfl_sync(0xffffffffu, beta, 0);
    t = __shfl_sync(0xffffffffu, t, 0);
    sc = __shfl_sync(0xffffffffu, sc, 0);
    for (int i = c + 1 + lane; i < n; i += 32) {
        const double v = (i == c + 1) ? 1.0 : col[i] * sc;
        vb[i] = v;
        gcol[i] = v;
    }
    if (lane == 0) {
        d[c] = col[c];
        e[c] = beta;
        tau[c] = t;
        scal[0] = t;
    }
}

__global__ void __launch_bounds__(SY_THREADS, 1)
    sytrd_cluster_kernel(const tnk_sytrd_sector* __restrict__ sec, double* __restrict__ G,
                         double* __restrict__ dv, double* __restrict__ ev,
                         double* __restrict__ tv) {
    cg::cluster_group cl = cg::this_cluster();
    const int cs = (int)cl.num_blocks();
    const int r = (int)cl.block_rank();
    const int s = blockIdx.x / cs;
    const int n = (int)sec[s].n;
    double* Gs = G + sec[s].g_off;
    double* d = dv + sec[s].v_off;
    double* e = ev + sec[s].v_off;
    double* tau = tv + sec[s].v_off;
    const int ncm = (n + cs - 1) / cs;
    const int ld = (int)sy_ld(n);
    const int ncl = r < n ? (n - r + cs - 1) / cs : 0;    // own columns j = r + cs * jl
    extern __shared__ double sh[];
    const SyShared S = sy_layout(sh, n, ncm);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    // own columns of the symmetric matrix from its lower triangle (column-major, ld n)
    for (int jl = 0; jl < ncl; ++jl) {
        const int j = r + cs * jl;
        for (int i = tid; i < n; i += SY_THREADS)
            S.A[(size_t)jl * ld + i] = i >= j ? Gs[(size_t)j * n + i] : Gs[(size_t)i * n + j];
    }
    __syncthreads();
    if (n >= 3 && r == 0 && warp == 0) householder_warp(S.A, 0, n, S.vb, Gs, d, e, tau, S.scal);

    for (int k = 0; k + 2 < n; ++k) {
        cl.sync();                                   // reflector k is in its owner's vb
        const int o = k % cs;
        // the reflector and its tau from the owner (independent remote loads, issued together)
        const double t = *cl.map_shared_rank(S.scal, o);
        {
            const double* rv = cl.map_shared_rank(S.vb, o);
            for (int i = k + 1 + tid; i < n; i += SY_THREADS) S.vl[i] = rv[i];
        }
        __syncthreads();
        // p_j = t A[:, j] . v (rows k+1 ..) for the na own columns j > k: thread (q, c) sums
        // the rows of chunk q of column c, then one thread per column adds the chunks
        const int jl0 = k >= r ? (k - r) / cs + 1 : 0;
        const int na = ncl - jl0;
        if (na > 0) {
            const int nq = min(SY_WARPS, max(1, SY_THREADS / na));
            const int m = n - k - 1;
            const int chunk = (m + nq - 1) / nq;
            if (tid < nq * na) {
                const int c = tid % na, q = tid / na;
                const double* col = S.A + (size_t)(jl0 + c) * ld;
                const int i1 = min(n, k + 1 + (q + 1) * chunk);
                double acc = 0.0;
                for (int i = k + 1 + q * chunk; i < i1; ++i) acc = fma(col[i], S.vl[i], acc);
                S.part[q * na + c] = acc;
            }
            __syncthreads();
            // warp 0 adds the chunks of every column (lanes c, c + 32), forms p_j and this CTA's
            // share of p . v; the cluster barrier below publishes them
            if (warp == 0) {
                double pv = 0.0;
                for (int c = lane; c < na; c += 32) {
                    double sum = 0.0;
                    for (int q = 0; q < nq; ++q) sum += S.part[q * na + c];
                    const double p = sum * t;
                    S.pown[jl0 + c] = p;
                    pv = fma(p, S.vl[r + cs * (jl0 + c)], pv);
                }
                pv = warp_sum(pv);
                if (lane == 0) S.scal[1] = pv;
            }
        } else if (tid == 0) {
            S.scal[1] = 0.0;
        }
        cl.sync();                                   // every p_j and share of p . v is written
        // the shares of p . v and this thread's p entries from the peers, loaded together
        double pv = lane < cs ? *cl.map_shared_rank(S.scal + 1, lane) : 0.0;
        constexpr int PG = 4;                        // p entries per thread per pass
        double pg[PG];
        int i0 = k + 1 + tid;
#pragma unroll
        for (int u = 0; u < PG; ++u) {
            const int i = i0 + u * SY_THREADS;
            pg[u] = i < n ? cl.map_shared_rank(S.pown, i % cs)[i / cs] : 0.0;
        }
        pv = warp_sum(pv);
        const double kc = 0.5 * t * pv;
        for (;;) {
#pragma unroll
            for (int u = 0; u < PG; ++u) {
                const int i = i0 + u * SY_THREADS;
                if (i < n) S.wl[i] = fma(-kc, S.vl[i], pg[u]);
            }
            i0 += PG * SY_THREADS;
            if (i0 >= n) break;
#pragma unroll
            for (int u = 0; u < PG; ++u) {
                const int i = i0 + u * SY_THREADS;
                pg[u] = i < n ? cl.map_shared_rank(S.pown, i % cs)[i / cs] : 0.0;
            }
        }
        __syncthreads();
        // A -= v w^T + w v^T on the own columns j > k. When column k + 1 is ours and still
        // needs a reflector, warp 0 updates it and forms that reflector while the other warps
        // update the rest (look-ahead: the next step's reflector is off the critical path).
        const int c = k + 1;
        const bool look = c + 2 < n && c % cs == r;
        const int jc = c / cs;
        if (look && warp == 0) {
            double* col = S.A + (size_t)jc * ld;
            const double vj = S.vl[c], wj = S.wl[c];
            for (int i = k + 1 + lane; i < n; i += 32)
                col[i] = fma(-S.vl[i], wj, fma(-S.wl[i], vj, col[i]));
            __syncwarp();
            householder_warp(col, c, n, S.vb, Gs + (size_t)c * n, d, e, tau, S.scal);
        } else {
            const int w0 = look ? 1 : 0, nw = SY_WARPS - w0;
            for (int jl = jl0 + warp - w0; jl < ncl; jl += nw) {
                if (look && jl == jc) continue;
                const int j = r + cs * jl;
                const double vj = S.vl[j], wj = S.wl[j];
                double* col = S.A + (size_t)jl * ld;
                for (int i = k + 1 + lane; i < n; i += 32)
                    col[i] = fma(-S.vl[i], wj, fma(-S.wl[i], vj, col[i]));
            }
        }
    }
    __syncthreads();
    // the trailing 2 x 2 (or 1 x 1) block
    if (tid == 0) {
        if (n >= 2 && (n - 2) % cs == r) {
            const double* col = S.A + (size_t)((n - 2) / cs) * ld;
            d[n - 2] = col[n - 2];
            e[n - 2] = col[n - 1];
            tau[n - 2] = 0.0;
        }
        if ((n - 1) % cs == r) d[n - 1] = S.A[(size_t)((n - 1) / cs) * ld + n - 1];
    }
    cl.sync();   // no CTA leaves while a peer may still read its shared memory
}

// Z (column-major n x k per sector, ld n) <- Q Z = H_0 H_1 ... H_{n-3} Z on the columns
// [col0, col0 + ncols) of one sector per CTA.
__global__ void __launch_bounds__(ORM_THREADS)
    ormtr_cols_kernel(const tnk_sytrd_sector* __restrict__ sec,
                      const tnk_ormtr_item* __restrict__ items, const double* __restrict__ G,
                      const double* __restrict__ tv, double* __restrict__ Z) {
    const tnk_ormtr_item it = items[blockIdx.x];
    const int n = (int)sec[it.sector].n;
    const double* Gs = G + sec[it.sector].g_off;
    const double* tau = tv + sec[it.sector].v_off;
    double* Zs = Z + sec[it.sector].z_off + (size_t)it.col0 * n;
    const int nc = it.ncols;
    extern __shared__ double sh[];
    double* zc = sh;                         // ORM_COLS columns of n
    double* vb = zc + (size_t)ORM_COLS * n;  // 2 x n
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int q = 0; q < nc; ++q)
        for (int i = tid; i < n; i += ORM_THREADS) zc[(size_t)q * n + i] = Zs[(size_t)q * n + i];
    for (int c = n - 3; c >= 0; --c) {
        double* v = vb + (size_t)(c & 1) * n;
        for (int i = c + 1 + tid; i < n; i += ORM_THREADS) v[i] = Gs[(size_t)c * n + i];
        __syncthreads();
        const double t = tau[c];
        if (t != 0.0 && warp < nc) {
            double* z = zc + (size_t)warp * n;
            double acc = 0.0;
            for (int i = c + 1 + lane; i < n; i += 32) acc = fma(v[i], z[i], acc);
            acc = -t * warp_sum(acc);
            for (int i = c + 1 + lane; i < n; i += 32) z[i] = fma(acc, v[i], z[i]);
        }
    }
    __syncthreads();
    for (int q = 0; q < nc; ++q)
        for (int i = tid; i < n; i += ORM_THREADS) Zs[(size_t)q * n + i] = zc[(size_t)q * n + i];
}

int max_optin_smem(int* bytes) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(bytes, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
            cudaSuccess) {
        tnk::set_error("sytrd: cannot query the device");
        return TNK_ERR_DEVICE;
    }
    return TNK_OK;
}

}  // namespace

extern "C" int tnk_sytrd_limits(int32_t cluster, int32_t* n_max) {
    if (!n_max || cluster < 1 || cluster > 16 || (cluster & (cluster - 1))) {
        tnk::set_error("tnk_sytrd_limits: cluster must be 1, 2, 4, 8 or 16");
        return TNK_ERR_ARG;
    }
    int smem = 0;
    int rc = max_optin_smem(&smem);
    if (rc) return rc;
    *n_max = 0;
    // clusters of this size must be launchable with one CTA of the largest shared memory per SM
    if (cluster > 8 &&
        cudaFuncSetAttribute(sytrd_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed,
                             1) != cudaSuccess) {
        cudaGetLastError();
        return TNK_OK;
    }
    if (cudaFuncSetAttribute(sytrd_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) != cudaSuccess) {
        cudaGetLastError();
        tnk::set_error("tnk_sytrd_limits: cannot raise the shared-memory limit");
        return TNK_ERR_CUDA;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(cluster);
    cfg.blockDim = dim3(SY_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int active = 0;
    if (cudaOccupancyMaxActiveClusters(&active, sytrd_cluster_kernel, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return TNK_OK;
    }
    if (active < 1) return TNK_OK;
    int64_t n = 1;
    while (8 * sy_shared_doubles(n + 1, cluster) <= smem) ++n;
    *n_max = (int32_t)n;
    return TNK_OK;
}

extern "C" int tnk_sytrd_batched_f64(const tnk_sytrd_sector* sectors, int32_t n_sectors,
                                     int32_t n_max, int32_t cluster, double* G, double* d,
                                     double* e, double* tau, void* stream) {
    if (n_sectors < 0 || (n_sectors && (!sectors || !G || !d || !e || !tau)) || n_max < 1 ||
        cluster < 1 || cluster > 16 || (cluster & (cluster - 1))) {
        tnk::set_error("tnk_sytrd_batched_f64: bad argument");
        return TNK_ERR_ARG;
    }
    if (n_sectors == 0) return TNK_OK;
    int smem = 0;
    int rc = max_optin_smem(&smem);
    if (rc) return rc;
    const int64_t need = 8 * sy_shared_doubles(n_max, cluster);
    if (need > smem) {
        tnk::set_error("tnk_sytrd_batched_f64: order %d needs %lld bytes of shared memory per "
                       "CTA with clusters of %d (the device has %d)",
                       n_max, (long long)need, cluster, smem);
        return TNK_ERR_SIZE;
    }
    if ((cluster > 8 &&
         cudaFuncSetAttribute(sytrd_cluster_kernel,
                              cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) ||
        cudaFuncSetAttribute(sytrd_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)need) != cudaSuccess) {
        cudaGetLastError();
        tnk::set_error("tnk_sytrd_batched_f64: cannot set the kernel's launch attributes");
        return TNK_ERR_CUDA;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)(n_sectors * cluster));
    cfg.blockDim = dim3(SY_THREADS);
    cfg.dynamicSmemBytes = need;
    cfg.stream = (cudaStream_t)stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, sytrd_cluster_kernel, sectors, G, d, e, tau) != cudaSuccess) {
        cudaError_t err = cudaGetLastError();
        tnk::set_error("sytrd_cluster_kernel: %s", cudaGetErrorString(err));
        return TNK_ERR_CUDA;
    }
    return TNK_OK;
}

extern "C" int tnk_ormtr_batched_f64(const tnk_sytrd_sector* sectors,
                                     const tnk_ormtr_item* items, int32_t n_items, int32_t n_max,
                                     const double* G, const double* tau, double* Z,
                                     void* stream) {
    if (n_items < 0 || (n_items && (!sectors || !items || !G || !tau || !Z)) || n_max < 1) {
        tnk::set_error("tnk_ormtr_batched_f64: bad argument");
        return TNK_ERR_ARG;
    }
    if (n_items == 0) return TNK_OK;
    int smem = 0;
    int rc = max_optin_smem(&smem);
    if (rc) return rc;
    const int64_t need = 8 * (int64_t)(ORM_COLS + 2) * n_max;
    if (need > smem) {
        tnk::set_error("tnk_ormtr_batched_f64: order %d needs %lld bytes of shared memory",
                       n_max, (long long)need);
        return TNK_ERR_SIZE;
    }
    if (cudaFuncSetAttribute(ormtr_cols_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)need) != cudaSuccess) {
        cudaGetLastError();
        tnk::set_error("tnk_ormtr_batched_f64: cannot set the shared-memory limit");
        return TNK_ERR_CUDA;
    }
    ormtr_cols_kernel<<<n_items, ORM_THREADS, need, (cudaStream_t)stream>>>(sectors, items, G,
                                                                             tau, Z);
    return tnk::check_launch("ormtr_cols_kernel");
}
