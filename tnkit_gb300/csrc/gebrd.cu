// The O(n^3) parts of the truncation's exact route on the device, for every charge sector of a
// bond in one launch each: the Householder bidiagonalisation A = Q_L B Q_R^T of each sector
// block (B upper bidiagonal), and, once the bidiagonal SVD B = U_B diag(s) V_B^T is known, the
// back-transformations U = Q_L U_B, V = Q_R V_B of the singular vectors the cut keeps. Together
// with the bidiagonal SVD between them (O(n^2) with deflation), this is the per-sector SVD that
// the truncation of tnkit/blocks.py:1380-1462 runs (method='svd', the reference's default,
// tnkit/blocks.py:1310-1344), as LAPACK's dgesdd does it (dgebrd, dbdsdc, dormbr).
//
// Bidiagonalisation (gebrd_cluster_kernel). One thread-block cluster per sector; the sector's
// m x n working matrix A (m >= n: the block or its transpose) stays in the distributed shared
// memory of its CTAs: CTA r holds the full columns j = r, r + CS, ... Step k (Golub and Van
// Loan, Matrix Computations, 4th ed., section 5.4.8):
//   left:  the owner of column k has formed H_k = I - tau_u u u^T (rows k .. m-1) that zeroes
//          column k below the diagonal (d_k = beta); every CTA copies u and applies H_k to its
//          own columns j > k (local: a dot product and an update per column);
//   right: row k's entries right of the diagonal are spread over the CTAs: each publishes the
//          sum of squares of its own entries (the owner of column k+1 also its alpha), every
//          CTA forms the reflector G_k = I - tau_v v v^T (columns k+1 .. n-1, e_k = beta) from
//          the same numbers in the same order and keeps v for its own columns; y = A[k+1:, k+1:] v
//          is summed over the cluster from unscaled parts published with the row norms (each CTA
//          one residue class of rows, then every CTA gathers the whole y), and every CTA
//          applies A -= tau_v y v^T to its columns;
//   the owner of column k + 1 applies both to that column first and forms H_{k+1} with one
//          warp while its other warps update (look-ahead).
// Three cluster barriers per step; no flag waits (every CTA of a cluster reaches every barrier
// the same number of times: the loop counts depend only on the sector's shape). Outputs: d, e,
// tau_u, tau_v per sector; reflector k's u (u[k] = 1 stored) in column k, rows k .. m-1, of the
// sector's m x n left-reflector matrix, v (v[k+1] = 1) in column k, rows k+1 .. n-1, of its
// n x n right-reflector matrix (both column-major).
//
// Back-transformation (ormqr_cols_kernel): Z <- H_0 H_1 ... H_{nr-1} Z for reflectors stored
// as above with their first row at k + shift (shift 0: left, 1: right); each CTA takes up to
// ORQ_COLS columns of one Z, keeps them in shared memory and applies the reflectors in turn.
#include <cooperative_groups.h>

#include "tnk_internal.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int GB_THREADS = 256;
constexpr int GB_WARPS = GB_THREADS / 32;
constexpr int ORQ_COLS = 8;
constexpr int ORQ_THREADS = ORQ_COLS * 32;

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__host__ __device__ inline int64_t gb_ld(int64_t m) { return m | 1; }

__host__ __device__ inline int64_t gb_shared_doubles(int64_t m, int64_t n, int cs) {
    const int64_t ncm = (n + cs - 1) / cs;
    return ncm * gb_ld(m) + 7 * m + 3 * ncm + GB_THREADS + 6;
}

struct GbShared {
    double* A;      // ncm columns of ld (the CTA's own columns, cyclic)
    double* ub;     // m: the left reflector this CTA formed (read by the peers)
    double* ul;     // m: the current left reflector
    double* yp;     // m: this CTA's part of y (read by the peers)
    double* yr;     // m: y summed over the cluster on this CTA's rows (read by the peers)
    double* yf;     // m: the whole y
    double* yc;     // m: column k + 1 when this CTA owns it (read by the peers)
    double* ycl;    // m: the owner's column k + 1 on this CTA's rows
    double* sown;   // ncm: the own columns' left dot products
    double* vown;   // ncm: the own entries of the right reflector
    double* xk;     // ncm: row k of the own columns, zero in column k + 1
    double* part;   // GB_THREADS: partial column dot products
    double* scal;   // 6: tau_u of ub, own sum of squares of row k, alpha of row k, tau_v, the
                    // right reflector's scale, spare
};

__device__ GbShared gb_layout(double* sh, int m, int ncm) {
    GbShared s;
    s.A = sh;
    s.ub = s.A + (size_t)ncm * gb_ld(m);
    s.ul = s.ub + m;
    s.yp = s.ul + m;
    s.yr = s.yp + m;
    s.yf = s.yr + m;
    s.yc = s.yf + m;
    s.ycl = s.yc + m;
    s.sown = s.ycl + m;
    s.vown = s.sown + ncm;
    s.xk = s.vown + ncm;
    s.part = s.xk + ncm;
    s.scal = s.part + GB_THREADS;
    return s;
}

// The left reflector of column c, formed by one warp from col (rows c .. m-1): H = I - tau u u^T
// with H [alpha; x] = [beta; 0], u = [1; x / (alpha - beta)] (tau = 0, u = e_1 when x = 0).
// Scalars on lane 0, broadcast. Writes u to ub and to column c of the left-reflector matrix
// (rows c .. m-1), tau to scal[0] and tau_u[c], d[c] = beta. The blocks are slices of a unit-norm
// two-site tensor, so their entries are at most 1 in magnitude and the sum of squares needs no
// scaling (it underflows only below 1e-154).
__device__ void left_house_warp(const double* col, int c, int m, double* ub, double* gcol,
                                double* d, double* tau_u, double* scal) {
    const int lane = threadIdx.x & 31;
    const double alpha = col[c];
    double ss = 0.0;
    for (int i = c + 1 + lane; i < m; i += 32) ss = fma(col[i], col[i], ss);
    ss = warp_sum_d(ss);
    double beta = alpha, t = 0.0, sc = 0.0;
    if (lane == 0 && ss > 0.0) {
        beta = -copysign(sqrt(fma(alpha, alpha, ss)), alpha);
        t = (beta - alpha) / beta;
        sc = 1.0 / (alpha - beta);
    }
    beta = __shfl_sync(0xffffffffu, beta, 0);
    t = __shfl_sync(0xffffffffu, t, 0);
    sc = __shfl_sync(0xffffffffu, sc, 0);
    for (int i = c + lane; i < m; i += 32) {
        const double u = (i == c) ? 1.0 : col[i] * sc;
        ub[i] = u;
        gcol[i] = u;
    }
    if (lane == 0) {
        d[c] = beta;
        tau_u[c] = t;
        scal[0] = t;
    }
}

__global__ void __launch_bounds__(GB_THREADS, 1)
    gebrd_cluster_kernel(const tnk_gebrd_sector* __restrict__ sec, const double* __restrict__ M,
                         double* __restrict__ UL, double* __restrict__ VR,
                         double* __restrict__ vec) {
    cg::cluster_group cl = cg::this_cluster();
    const int cs = (int)cl.num_blocks();
    const int r = (int)cl.block_rank();
    const tnk_gebrd_sector sd = sec[blockIdx.x / cs];
    const int m = (int)sd.m, n = (int)sd.n;
    const double* As = M + sd.a_off;
    double* ULs = UL + sd.ul_off;       // m x n, column-major
    double* VRs = VR + sd.vr_off;       // n x n, column-major
    double* d = vec + sd.v_off;
    double* e = d + n;
    double* tau_u = e + n;
    double* tau_v = tau_u + n;
    const int ncm = (n + cs - 1) / cs;
    const int ld = (int)gb_ld(m);
    const int ncl = r < n ? (n - r + cs - 1) / cs : 0;    // own columns j = r + cs * jl
    extern __shared__ double sh[];
    const GbShared S = gb_layout(sh, m, ncm);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    for (int jl = 0; jl < ncl; ++jl) {
        const int j = r + cs * jl;
        for (int i = tid; i < m; i += GB_THREADS)
            S.A[(size_t)jl * ld + i] = As[(int64_t)i * sd.a_rs + (int64_t)j * sd.a_cs];
    }
    __syncthreads();
    if (r == 0 && warp == 0) left_house_warp(S.A, 0, m, S.ub, ULs, d, tau_u, S.scal);

    for (int k = 0; k < n; ++k) {
        cl.sync();                                   // (1) H_k is in its owner's ub
        const int o = k % cs;
        const double tu = *cl.map_shared_rank(S.scal, o);
        {
            const double* rv = cl.map_shared_rank(S.ub, o);
            for (int i = k + tid; i < m; i += GB_THREADS) S.ul[i] = rv[i];
        }
        __syncthreads();
        // left: s_j = tau_u u . A[k:, j] for the na own columns j > k (row chunks, then one
        // warp adds the chunks), then A[k:, j] -= s_j u
        const int jl0 = k >= r ? (k - r) / cs + 1 : 0;
        const int na = ncl - jl0;
        if (na > 0) {
            const int nq = min(GB_WARPS, max(1, GB_THREADS / na));
            const int rows = m - k;
            const int chunk = (rows + nq - 1) / nq;
            if (tid < nq * na) {
                const int c = tid % na, q = tid / na;
                const double* col = S.A + (size_t)(jl0 + c) * ld;
                const int i1 = min(m, k + (q + 1) * chunk);
                double acc = 0.0;
                for (int i = k + q * chunk; i < i1; ++i) acc = fma(col[i], S.ul[i], acc);
                S.part[q * na + c] = acc;
            }
            __syncthreads();
            if (warp == 0) {
                for (int c = lane; c < na; c += 32) {
                    double sum = 0.0;
                    for (int q = 0; q < nq; ++q) sum += S.part[q * na + c];
                    S.sown[jl0 + c] = sum * tu;
                }
            }
            __syncthreads();
            for (int jl = jl0 + warp; jl < ncl; jl += GB_WARPS) {
                const double s = S.sown[jl];
                double* col = S.A + (size_t)jl * ld;
                for (int i = k + lane; i < m; i += 32) col[i] = fma(-s, S.ul[i], col[i]);
            }
        }
        if (k + 1 >= n) break;                       // (uniform over the cluster)
        __syncthreads();
        if (k + 2 >= n) {
            // the last superdiagonal entry needs no reflector; column k + 1 still gets its
            // left reflector (rows k+1 .. m-1) from its owner
            if ((k + 1) % cs == r) {
                const int jc = (k + 1) / cs;
                if (tid == 0) {
                    e[k] = S.A[(size_t)jc * ld + k];
                    tau_v[k] = 0.0;
                }
                if (warp == 0)
                    left_house_warp(S.A + (size_t)jc * ld, k + 1, m, S.ub,
                                    ULs + (size_t)(k + 1) * m, d, tau_u, S.scal);
            }
            continue;                                // next step: barrier (1), left only
        }
        // right: G_k's vector is v = sc x + e_{k+1} with x the row k entries right of column
        // k + 1 and sc known only once the row's norm is, so y = A v is gathered unscaled: each
        // CTA's x part yp (own columns j > k + 1) and, from the owner of column k + 1, that
        // column yc; y = sc sum(yp) + yc. Here: own sum of squares of x, alpha = A[k][k+1], yp,
        // and yc (owner of k + 1).
        const bool own1 = (k + 1) % cs == r;
        const int j1 = own1 ? (k + 1) / cs : -1;
        if (warp == 0) {
            double ss = 0.0;
            for (int jl = jl0 + lane; jl < ncl; jl += 32) {
                const double a = S.A[(size_t)jl * ld + k];
                const double x = jl == j1 ? 0.0 : a;         // x: row k without column k + 1
                S.xk[jl] = x;
                ss = fma(x, x, ss);
            }
            ss = warp_sum_d(ss);
            if (lane == 0) {
                S.scal[1] = ss;
                if (own1) S.scal[2] = S.A[(size_t)j1 * ld + k];
            }
        }
        __syncthreads();
        for (int i = k + 1 + tid; i < m; i += GB_THREADS) {
            double acc = 0.0;
            for (int jl = jl0; jl < ncl; ++jl) acc = fma(S.A[(size_t)jl * ld + i], S.xk[jl], acc);
            S.yp[i] = acc;
            if (own1) S.yc[i] = S.A[(size_t)j1 * ld + i];
        }
        cl.sync();                                   // (2) row norms and y parts are published
        if (warp == 0) {
            // every CTA forms the same reflector from the same numbers in the same order
            double ss = lane < cs ? *cl.map_shared_rank(S.scal + 1, lane) : 0.0;
            const double alpha = *cl.map_shared_rank(S.scal + 2, (k + 1) % cs);
            ss = warp_sum_d(ss);
            if (lane == 0) {
                double beta = alpha, tv = 0.0, sc = 0.0;
                if (ss > 0.0) {
                    // one division: q = 1 / (beta (alpha - beta)) gives 1/beta = (alpha - beta) q
                    // and 1/(alpha - beta) = beta q
                    beta = -copysign(sqrt(fma(alpha, alpha, ss)), alpha);
                    const double am = alpha - beta;
                    const double ba = beta * am;
                    if (fabs(ba) > 1e-290) {
                        const double q = 1.0 / ba;
                        tv = -am * am * q;
                        sc = beta * q;
                    } else {                                 // (entries below ~1e-145)
                        tv = (beta - alpha) / beta;
                        sc = 1.0 / am;
                    }
                }
                if (r == 0) {
                    e[k] = beta;
                    tau_v[k] = tv;
                }
                S.scal[3] = tv;
                S.scal[4] = sc;
            }
        }
        // meanwhile the unscaled sums of this CTA's residue class of rows (all peers' loads in
        // flight at once, summed in rank order) and the owner's column k + 1 there
        for (int i = k + 1 + r + cs * tid; i < m; i += cs * GB_THREADS) {
            double part[16];
#pragma unroll
            for (int q = 0; q < 16; ++q) part[q] = q < cs ? cl.map_shared_rank(S.yp, q)[i] : 0.0;
            const double c1 = cl.map_shared_rank(S.yc, (k + 1) % cs)[i];
            double acc = 0.0;
#pragma unroll
            for (int q = 0; q < 16; ++q) acc += part[q];
            S.yr[i] = acc;
            S.ycl[i] = c1;
        }
        __syncthreads();
        const double tv = S.scal[3];
        const double sc = S.scal[4];
        for (int i = k + 1 + r + cs * tid; i < m; i += cs * GB_THREADS)
            S.yr[i] = fma(sc, S.yr[i], S.ycl[i]);
        for (int jl = jl0 + tid; jl < ncl; jl += GB_THREADS) {
            const int j = r + cs * jl;
            const double v = (j == k + 1) ? 1.0 : S.A[(size_t)jl * ld + k] * sc;
            S.vown[jl] = v;
            VRs[(size_t)k * n + j] = v;
        }
        cl.sync();                                   // (3) y is summed, by residue class
        for (int i = k + 1 + tid; i < m; i += GB_THREADS)
            S.yf[i] = cl.map_shared_rank(S.yr, (i - k - 1) % cs)[i];
        __syncthreads();
        // A[k+1:, j] -= tau_v y v_j; column k + 1 first when it is ours: warp 0 updates it and
        // forms H_{k+1} while the other warps update the rest
        const int c = k + 1;
        const bool look = c % cs == r;
        const int jc = c / cs;
        if (look && warp == 0) {
            double* col = S.A + (size_t)jc * ld;
            const double f = tv * S.vown[jc];
            for (int i = k + 1 + lane; i < m; i += 32) col[i] = fma(-f, S.yf[i], col[i]);
            __syncwarp();
            left_house_warp(col, c, m, S.ub, ULs + (size_t)c * m, d, tau_u, S.scal);
        } else {
            const int w0 = look ? 1 : 0, nw = GB_WARPS - w0;
            for (int jl = jl0 + warp - w0; jl < ncl; jl += nw) {
                if (look && jl == jc) continue;
                const double f = tv * S.vown[jl];
                double* col = S.A + (size_t)jl * ld;
                for (int i = k + 1 + lane; i < m; i += 32) col[i] = fma(-f, S.yf[i], col[i]);
            }
        }
    }
    cl.sync();   // no CTA leaves while a peer may still read its shared memory
}

// Z <- H_0 H_1 ... H_{nr-1} Z on columns [col0, col0 + ncols) of one reflector set per CTA.
__global__ void __launch_bounds__(ORQ_THREADS)
    ormqr_cols_kernel(const tnk_refl_set* __restrict__ sets,
                      const tnk_ormtr_item* __restrict__ items, const double* __restrict__ R,
                      const double* __restrict__ tau, double* __restrict__ Z) {
    const tnk_ormtr_item it = items[blockIdx.x];
    const tnk_refl_set st = sets[it.sector];
    const int rows = (int)st.rows, nr = (int)st.nrefl, sh = st.shift;
    const double* Rs = R + st.r_off;
    const double* ts = tau + st.tau_off;
    double* Zs = Z + st.z_off + (size_t)it.col0 * rows;
    const int nc = it.ncols;
    extern __shared__ double smem[];
    double* zc = smem;                          // ORQ_COLS columns of rows
    double* vb = zc + (size_t)ORQ_COLS * rows;  // 2 x rows
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int q = 0; q < nc; ++q)
        for (int i = tid; i < rows; i += ORQ_THREADS)
            zc[(size_t)q * rows + i] = Zs[(size_t)q * rows + i];
    for (int c = nr - 1; c >= 0; --c) {
        const int f = c + sh;                   // first row of reflector c
        double* v = vb + (size_t)(c & 1) * rows;
        for (int i = f + tid; i < rows; i += ORQ_THREADS) v[i] = Rs[(size_t)c * rows + i];
        __syncthreads();
        const double t = ts[c];
        if (t != 0.0 && warp < nc && f < rows) {
            double* z = zc + (size_t)warp * rows;
            double acc = 0.0;
            for (int i = f + lane; i < rows; i += 32) acc = fma(v[i], z[i], acc);
            acc = -t * warp_sum_d(acc);
            for (int i = f + lane; i < rows; i += 32) z[i] = fma(acc, v[i], z[i]);
        }
    }
    __syncthreads();
    for (int q = 0; q < nc; ++q)
        for (int i = tid; i < rows; i += ORQ_THREADS)
            Zs[(size_t)q * rows + i] = zc[(size_t)q * rows + i];
}

int max_smem(int* bytes) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(bytes, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
            cudaSuccess) {
        tnk::set_error("gebrd: cannot query the device");
        return TNK_ERR_DEVICE;
    }
    return TNK_OK;
}

}  // namespace

extern "C" int tnk_gebrd_limits(int32_t cluster, int32_t* m_max) {
    if (!m_max || cluster < 1 || cluster > 16 || (cluster & (cluster - 1))) {
        tnk::set_error("tnk_gebrd_limits: cluster must be 1, 2, 4, 8 or 16");
        return TNK_ERR_ARG;
    }
    int smem = 0;
    int rc = max_smem(&smem);
    if (rc) return rc;
    *m_max = 0;
    if (cluster > 8 &&
        cudaFuncSetAttribute(gebrd_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed,
                             1) != cudaSuccess) {
        cudaGetLastError();
        return TNK_OK;
    }
    if (cudaFuncSetAttribute(gebrd_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) != cudaSuccess) {
        cudaGetLastError();
        tnk::set_error("tnk_gebrd_limits: cannot raise the shared-memory limit");
        return TNK_ERR_CUDA;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(cluster);
    cfg.blockDim = dim3(GB_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int active = 0;
    if (cudaOccupancyMaxActiveClusters(&active, gebrd_cluster_kernel, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return TNK_OK;
    }
    if (active < 1) return TNK_OK;
    int64_t mm = 1;    // the largest square m x m block that fits (m >= n)
    while (8 * gb_shared_doubles(mm + 1, mm + 1, cluster) <= smem) ++mm;
    *m_max = (int32_t)mm;
    return TNK_OK;
}

extern "C" int tnk_gebrd_batched_f64(const tnk_gebrd_sector* sectors, int32_t n_sectors,
                                     int32_t m_max, int32_t n_max, int32_t cluster,
                                     const double* M, double* UL, double* VR, double* vec,
                                     void* stream) {
    if (n_sectors < 0 || (n_sectors && (!sectors || !M || !UL || !VR || !vec)) || m_max < 1 ||
        n_max < 1 || n_max > m_max || cluster < 1 || cluster > 16 ||
        (cluster & (cluster - 1))) {
        tnk::set_error("tnk_gebrd_batched_f64: bad argument");
        return TNK_ERR_ARG;
    }
    if (n_sectors == 0) return TNK_OK;
    int smem = 0;
    int rc = max_smem(&smem);
    if (rc) return rc;
    const int64_t need = 8 * gb_shared_doubles(m_max, n_max, cluster);
    if (need > smem) {
        tnk::set_error("tnk_gebrd_batched_f64: a %d x %d block needs %lld bytes of shared "
                       "memory per CTA with clusters of %d (the device has %d)",
                       m_max, n_max, (long long)need, cluster, smem);
        return TNK_ERR_SIZE;
    }
    if ((cluster > 8 &&
         cudaFuncSetAttribute(gebrd_cluster_kernel,
                              cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) ||
        cudaFuncSetAttribute(gebrd_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)need) != cudaSuccess) {
        cudaGetLastError();
        tnk::set_error("tnk_gebrd_batched_f64: cannot set the kernel's launch attributes");
        return TNK_ERR_CUDA;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)(n_sectors * cluster));
    cfg.blockDim = dim3(GB_THREADS);
    cfg.dynamicSmemBytes = need;
    cfg.stream = (cudaStream_t)stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, gebrd_cluster_kernel, sectors, M, UL, VR, vec) != cudaSuccess) {
        cudaError_t err = cudaGetLastError();
        tnk::set_error("gebrd_cluster_kernel: %s", cudaGetErrorString(err));
        return TNK_ERR_CUDA;
    }
    return TNK_OK;
}

extern "C" int tnk_ormqr_batched_f64(const tnk_refl_set* sets, const tnk_ormtr_item* items,
                                     int32_t n_items, int32_t rows_max, const double* R,
                                     const double* tau, double* Z, void* stream) {
    if (n_items < 0 || (n_items && (!sets || !items || !R || !tau || !Z)) || rows_max < 1) {
        tnk::set_error("tnk_ormqr_batched_f64: bad argument");
        return TNK_ERR_ARG;
    }
    if (n_items == 0) return TNK_OK;
    int smem = 0;
    int rc = max_smem(&smem);
    if (rc) return rc;
    const int64_t need = 8 * (int64_t)(ORQ_COLS + 2) * rows_max;
    if (need > smem) {
        tnk::set_error("tnk_ormqr_batched_f64: %d rows need %lld bytes of shared memory",
                       rows_max, (long long)need);
        return TNK_ERR_SIZE;
    }
    if (cudaFuncSetAttribute(ormqr_cols_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)need) != cudaSuccess) {
        cudaGetLastError();
        tnk::set_error("tnk_ormqr_batched_f64: cannot set the shared-memory limit");
        return TNK_ERR_CUDA;
    }
    ormqr_cols_kernel<<<n_items, ORQ_THREADS, need, (cudaStream_t)stream>>>(sets, items, R, tau,
                                                                            Z);
    return tnk::check_launch("ormqr_cols_kernel");
}
