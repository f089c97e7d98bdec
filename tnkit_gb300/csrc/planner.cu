// Host planner (no device code): the block tables of the one- and two-site H_eff contraction,
// built from the layouts' sector keys in one pass, and their re-layout for the tensor-core
// path. The tables are those of the three-stage plan (include/tnkit_gb300.h):
//
//   stage 1  Y[(a', w), (s.., b)] = L[(a', w), a] theta[a, (s.., b)]     one GEMM per pair of
//            an L block and a theta block that share the sector of a
//   stage 2  Z[(a', s'.., r), b] = sum_{w, s..} S[w, s.., s'.., r] Y[...]  combination with the
//            nonzero entries of the combined MPO S, one task per (s'.., r) slice of a Z block
//   stage 3  out[(a', s'..), b'] = sum_{r, b} Z[(a', s'..), (r, b)] R[b', (r, b)]
//
// The reference pairs matching blocks in Python at every tensordot of its matvec
// (tnkit/blocks.py:1089-1090); here the pairing, the MPO coefficients and the workspace
// offsets are worked out once per local problem. The Python planner (plan.py) states the same
// construction and the tests require identical tables from both.
#include <algorithm>
#include <array>
#include <climits>
#include <cmath>
#include <map>
#include <new>
#include <stdexcept>
#include <unordered_map>
#include <utility>
#include <vector>

#include "tnk_internal.cuh"

namespace {

struct PlanBuild {
    std::vector<tnk_gemm_task> g1t, g3t, t1, t3;
    std::vector<tnk_gemm_seg> g1s, g3s;
    std::vector<tnk_comb_task> c2t, t2;
    std::vector<tnk_comb_term> c2c;
    std::vector<tnk_tc_seg> s1, s3;
    std::vector<int64_t> maps;                 // (offset, rows, cols, ld) per tensor map
    std::vector<tnk_cvt_task> cvt[3];          // staging of L, R, theta
    int64_t ws1 = 0, ws2 = 0, macs1 = 0, macs3 = 0, cursor = 0;
};

struct Lay {
    const tnk_layout_desc* d;
    int64_t key(int64_t b, int l) const { return d->keys[b * d->nlegs + l]; }
    int64_t shape(int64_t b, int l) const { return d->shapes[b * d->nlegs + l]; }
    int64_t off(int64_t b) const { return d->offsets[b]; }
    int64_t nb() const { return d->nblocks; }
};

constexpr int SLOT_X0 = 0, SLOT_X1 = 1, SLOT_X2 = 2, SLOT_WS = 3;

bool fits32(int64_t v) { return v >= INT_MIN && v <= INT_MAX; }

struct Overflow {};

int32_t i32(int64_t v) {
    if (!fits32(v)) throw Overflow{};
    return (int32_t)v;
}

tnk_gemm_seg make_seg(int64_t a_off, int64_t a_rs, int64_t a_cs, int a_buf, int64_t b_off,
                      int64_t b_rs, int64_t b_cs, int b_buf, int64_t k) {
    tnk_gemm_seg s{};
    s.a_off = a_off;
    s.b_off = b_off;
    s.a_rs = i32(a_rs);
    s.a_cs = i32(a_cs);
    s.b_rs = i32(b_rs);
    s.b_cs = i32(b_cs);
    s.k = i32(k);
    s.a_buf = (int16_t)a_buf;
    s.b_buf = (int16_t)b_buf;
    s.conj = 0;
    s.pad = 0;
    s.coef = 1.0;
    return s;
}

tnk_gemm_task make_task(int64_t c_off, int64_t ldc, int64_t m, int64_t n, int64_t b, int64_t e,
                        int flags) {
    tnk_gemm_task t{};
    t.c_off = c_off;
    t.ldc = i32(ldc);
    t.m = i32(m);
    t.n = i32(n);
    t.seg_begin = i32(b);
    t.seg_end = i32(e);
    t.flags = flags;
    return t;
}

// (a', w, s_1 [, s_2], b) sector indices of a stage-1 output block; unused entries -1
using YKey = std::array<int64_t, 5>;

struct Slice {
    YKey yk;
    int64_t wsec, rsec, isec[2], osec[2];
};

struct ZDef {
    int64_t P, PO, Rd, B, kr;
    int64_t osec[2];
    std::vector<Slice> slices;
};

int apply_build(const tnk_apply_plan_in* in, PlanBuild* pb) {
    const int n = in->n_sites;
    if (n != 1 && n != 2) {
        tnk::set_error("plan_apply: one or two sites, got %d", n);
        return TNK_ERR_ARG;
    }
    const Lay th{&in->theta}, L{&in->L}, R{&in->R}, out{&in->out};
    if (in->theta.nlegs != n + 2 || in->L.nlegs != 3 || in->R.nlegs != 3 ||
        in->out.nlegs != n + 2 || !in->S || !in->sec_start || !in->sec_dim) {
        tnk::set_error("plan_apply: bad layout descriptors");
        return TNK_ERR_ARG;
    }
    const int ax = 2 * n + 2;
    int64_t st[6];
    st[ax - 1] = 1;
    for (int a = ax - 2; a >= 0; --a) st[a] = st[a + 1] * in->s_dims[a + 1];
    auto nsec = [&](int a) { return in->sec_begin[a + 1] - in->sec_begin[a]; };
    auto sstart = [&](int a, int64_t s) { return in->sec_start[in->sec_begin[a] + s]; };
    auto sdim = [&](int a, int64_t s) { return in->sec_dim[in->sec_begin[a] + s]; };
    auto sector_ok = [&](int a, int64_t s) { return s >= 0 && s < nsec(a); };

    // S entry of a slice at (ww, pi, po, rr): pi / po flatten the in / out sector dims (C order)
    auto value = [&](const Slice& sl, int64_t ww, int64_t pi, int64_t po, int64_t rr) {
        int64_t idx = (sstart(0, sl.wsec) + ww) * st[0] + (sstart(ax - 1, sl.rsec) + rr) * st[ax - 1];
        for (int a = n - 1; a >= 0; --a) {
            const int64_t di = sdim(1 + a, sl.isec[a]), dO = sdim(1 + n + a, sl.osec[a]);
            idx += (sstart(1 + a, sl.isec[a]) + pi % di) * st[1 + a];
            idx += (sstart(1 + n + a, sl.osec[a]) + po % dO) * st[1 + n + a];
            pi /= di;
            po /= dO;
        }
        return in->S[idx];
    };
    auto prod_in = [&](const Slice& sl) {
        int64_t p = 1;
        for (int a = 0; a < n; ++a) p *= sdim(1 + a, sl.isec[a]);
        return p;
    };
    auto prod_out = [&](const Slice& sl) {
        int64_t p = 1;
        for (int a = 0; a < n; ++a) p *= sdim(1 + n + a, sl.osec[a]);
        return p;
    };
    auto any_nonzero = [&](const Slice& sl) {
        const int64_t wd = sdim(0, sl.wsec), rd = sdim(ax - 1, sl.rsec);
        const int64_t pin = prod_in(sl), pon = prod_out(sl);
        for (int64_t ww = 0; ww < wd; ++ww)
            for (int64_t pi = 0; pi < pin; ++pi)
                for (int64_t po = 0; po < pon; ++po)
                    for (int64_t rr = 0; rr < rd; ++rr)
                        if (value(sl, ww, pi, po, rr) != 0.0) return true;
        return false;
    };

    std::unordered_map<int64_t, std::vector<int64_t>> th_by_q, r_by_d;
    for (int64_t k = 0; k < th.nb(); ++k) th_by_q[th.key(k, 0)].push_back(k);
    for (int64_t k = 0; k < R.nb(); ++k) r_by_d[R.key(k, 0)].push_back(k);
    std::map<YKey, std::pair<int64_t, int64_t>> ycand;
    std::map<std::pair<int64_t, int64_t>, std::vector<YKey>> y_by_pb;
    for (int64_t kl = 0; kl < L.nb(); ++kl) {
        auto it = th_by_q.find(L.key(kl, 2));
        if (it == th_by_q.end()) continue;
        for (int64_t kt : it->second) {
            YKey yk{L.key(kl, 0), L.key(kl, 1), -1, -1, -1};
            for (int a = 0; a < n; ++a) yk[2 + a] = th.key(kt, 1 + a);
            yk[2 + n] = th.key(kt, n + 1);
            ycand[yk] = {kl, kt};
            y_by_pb[{L.key(kl, 0), th.key(kt, n + 1)}].push_back(yk);
        }
    }

    std::vector<ZDef> zdefs;
    std::vector<std::pair<int64_t, std::vector<int64_t>>> tasks3;
    for (int64_t ko = 0; ko < out.nb(); ++ko) {
        const int64_t p = out.key(ko, 0), d = out.key(ko, n + 1), P = out.shape(ko, 0);
        int64_t PO = 1;
        for (int a = 0; a < n; ++a) PO *= out.shape(ko, 1 + a);
        std::vector<int64_t> segs3;
        auto rit = r_by_d.find(d);
        if (rit != r_by_d.end()) {
            for (int64_t kr : rit->second) {
                const int64_t r = R.key(kr, 1), b = R.key(kr, 2);
                auto yit = y_by_pb.find({p, b});
                if (yit == y_by_pb.end()) continue;
                std::vector<Slice> slices;
                for (const YKey& yk : yit->second) {
                    Slice sl{};
                    sl.yk = yk;
                    sl.wsec = yk[1];
                    sl.rsec = r;
                    for (int a = 0; a < n; ++a) {
                        sl.isec[a] = yk[2 + a];
                        sl.osec[a] = out.key(ko, 1 + a);
                    }
                    bool ok = sector_ok(0, sl.wsec) && sector_ok(ax - 1, sl.rsec);
                    for (int a = 0; a < n; ++a)
                        ok = ok && sector_ok(1 + a, sl.isec[a]) && sector_ok(1 + n + a, sl.osec[a]);
                    if (!ok) {
                        tnk::set_error("plan_apply: a block key names a sector the MPO lacks");
                        return TNK_ERR_ARG;
                    }
                    if (any_nonzero(sl)) slices.push_back(sl);
                }
                if (slices.empty()) continue;
                ZDef z{};
                z.P = P;
                z.PO = PO;
                z.Rd = R.shape(kr, 1);
                z.B = R.shape(kr, 2);
                z.kr = kr;
                for (int a = 0; a < n; ++a) z.osec[a] = out.key(ko, 1 + a);
                z.slices = std::move(slices);
                zdefs.push_back(std::move(z));
                segs3.push_back((int64_t)zdefs.size() - 1);
            }
        }
        tasks3.emplace_back(ko, std::move(segs3));
    }

    // stage 1: the Y blocks some Z block uses, in order of first use
    std::map<YKey, int64_t> y_off;
    for (const ZDef& z : zdefs)
        for (const Slice& sl : z.slices) {
            if (y_off.count(sl.yk)) continue;
            const auto [kl, kt] = ycand.at(sl.yk);
            const int64_t P = L.shape(kl, 0), Wd = L.shape(kl, 1), Q = L.shape(kl, 2);
            int64_t ncols = 1;
            for (int a = 1; a <= n + 1; ++a) ncols *= th.shape(kt, a);
            y_off[sl.yk] = pb->ws1;
            const int64_t b = (int64_t)pb->g1s.size();
            pb->g1s.push_back(make_seg(L.off(kl), Q, 1, SLOT_X0, th.off(kt), ncols, 1, SLOT_X1, Q));
            pb->g1t.push_back(make_task(pb->ws1, ncols, P * Wd, ncols, b, b + 1, 0));
            pb->macs1 += P * Wd * ncols * Q;
            pb->ws1 += P * Wd * ncols;
        }

    // stage 2: one combination task per (s'.., r) slice of every Z block
    std::vector<int64_t> z_off;
    z_off.reserve(zdefs.size());
    for (const ZDef& z : zdefs) {
        const int64_t base = pb->ws1 + pb->ws2;
        z_off.push_back(base);
        pb->ws2 += z.P * z.PO * z.Rd * z.B;
        const int64_t ld = z.PO * z.Rd * z.B;
        const int64_t po_n = prod_out(z.slices[0]);
        struct Prep {
            int64_t yo, src_ld, ncols, Wd, pi_n;
            const Slice* sl;
        };
        std::vector<Prep> preps;
        for (const Slice& sl : z.slices) {
            const auto [kl, kt] = ycand.at(sl.yk);
            int64_t ncols = 1, pi_n = 1;
            for (int a = 1; a <= n + 1; ++a) ncols *= th.shape(kt, a);
            for (int a = 1; a <= n; ++a) pi_n *= th.shape(kt, a);
            const int64_t Wd = L.shape(kl, 1);
            preps.push_back({y_off.at(sl.yk), Wd * ncols, ncols, Wd, pi_n, &sl});
        }
        for (int64_t po = 0; po < po_n; ++po)
            for (int64_t rr = 0; rr < z.Rd; ++rr) {
                const int64_t dst = base + (po * z.Rd + rr) * z.B;
                const int64_t tb = (int64_t)pb->c2c.size();
                for (const Prep& q : preps)
                    for (int64_t ww = 0; ww < q.Wd; ++ww)
                        for (int64_t pi = 0; pi < q.pi_n; ++pi) {
                            const double v = value(*q.sl, ww, pi, po, rr);
                            if (v == 0.0) continue;
                            tnk_comb_term t{};
                            t.src_off = q.yo + ww * q.ncols + pi * z.B;
                            t.src_ld = i32(q.src_ld);
                            t.src_cs = 1;
                            t.coef = v;
                            pb->c2c.push_back(t);
                        }
                tnk_comb_task c{};
                c.dst_off = dst;
                c.rows = i32(z.P);
                c.cols = i32(z.B);
                c.dst_ld = i32(ld);
                c.dst_cs = 1;
                c.term_begin = i32(tb);
                c.term_end = i32((int64_t)pb->c2c.size());
                pb->c2t.push_back(c);
            }
    }

    // stage 3: every output block from its Z blocks and R blocks
    for (const auto& [ko, segs3] : tasks3) {
        const int64_t P = out.shape(ko, 0), D = out.shape(ko, n + 1);
        int64_t PO = 1;
        for (int a = 0; a < n; ++a) PO *= out.shape(ko, 1 + a);
        const int64_t b = (int64_t)pb->g3s.size();
        for (int64_t zi : segs3) {
            const ZDef& z = zdefs[zi];
            const int64_t K = z.Rd * z.B;
            pb->g3s.push_back(make_seg(z_off[zi], K, 1, SLOT_WS, R.off(z.kr), 1, K, SLOT_X2, K));
            pb->macs3 += P * PO * D * K;
        }
        pb->g3t.push_back(make_task(out.off(ko), D, P * PO, D, b, (int64_t)pb->g3s.size(), 0));
    }
    return TNK_OK;
}

constexpr int64_t TC_ALIGN = 32;   // staged block bases: 32 floats = 128 bytes

int64_t rup(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

int tc_build(const tnk_gemm_task* t1, int64_t nt1, const tnk_gemm_seg* s1,
             const tnk_comb_task* t2, int64_t nt2, const tnk_gemm_task* t3, int64_t nt3,
             const tnk_gemm_seg* s3, PlanBuild* pb) {
    enum { KL = 0, KR = 1, KT = 2, KZ = 3 };
    std::map<std::pair<int, int64_t>, int64_t> map_of;
    auto staged = [&](int kind, int64_t src_off, int64_t rows, int64_t cols, bool transpose) {
        auto it = map_of.find({kind, src_off});
        if (it != map_of.end()) return it->second;
        const int64_t r = transpose ? cols : rows, c = transpose ? rows : cols;
        const int64_t ld = rup(c, 4);
        const int64_t off = pb->cursor;
        pb->cursor += rup(r * ld, TC_ALIGN);
        if (kind != KZ) {
            tnk_cvt_task cv{};
            cv.src_off = src_off;
            cv.dst_off = off;
            cv.rows = i32(rows);
            cv.cols = i32(cols);
            cv.src_ld = i32(cols);
            cv.dst_ld = i32(ld);
            cv.transpose = transpose ? 1 : 0;
            cv.pad = 0;
            pb->cvt[kind].push_back(cv);
        }
        const int64_t idx = (int64_t)pb->maps.size() / 4;
        pb->maps.insert(pb->maps.end(), {off, r, c, ld});
        map_of[{kind, src_off}] = idx;
        return idx;
    };
    auto tc_seg = [](int64_t am, int64_t bm, int64_t k) {
        tnk_tc_seg s{};
        s.a_map = i32(am);
        s.b_map = i32(bm);
        s.k = i32(k);
        s.pad = 0;
        return s;
    };
    // stage 1: A = L block (m x k), B = theta block (k x n) staged transposed (n x k)
    for (int64_t i = 0; i < nt1; ++i) {
        const tnk_gemm_task& t = t1[i];
        const int64_t b = (int64_t)pb->s1.size();
        for (int64_t j = t.seg_begin; j < t.seg_end; ++j) {
            const int64_t am = staged(KL, s1[j].a_off, t.m, s1[j].k, false);
            const int64_t bm = staged(KT, s1[j].b_off, s1[j].k, t.n, true);
            pb->s1.push_back(tc_seg(am, bm, s1[j].k));
        }
        pb->t1.push_back(make_task(t.c_off, t.ldc, t.m, t.n, b, (int64_t)pb->s1.size(), 0));
    }
    // Z blocks (stage-3 A operands), keyed by their FP64 workspace offset
    std::map<int64_t, std::array<int64_t, 3>> zinfo;   // offset -> (K, M, map)
    for (int64_t i = 0; i < nt3; ++i)
        for (int64_t j = t3[i].seg_begin; j < t3[i].seg_end; ++j) {
            const int64_t zo = s3[j].a_off;
            if (zinfo.count(zo)) continue;
            const int64_t K = s3[j].k, M = t3[i].m;
            zinfo[zo] = {K, M, staged(KZ, zo, M, K, false)};
        }
    // stage 2: destinations remapped into the padded Z blocks
    for (int64_t i = 0; i < nt2; ++i) {
        const tnk_comb_task& t = t2[i];
        auto it = zinfo.upper_bound(t.dst_off);
        if (it == zinfo.begin()) {
            tnk::set_error("plan_tc: a stage-2 destination precedes every Z block");
            return TNK_ERR_ARG;
        }
        --it;
        const int64_t zo = it->first, K = it->second[0], mi = it->second[2];
        const int64_t off = pb->maps[4 * mi], ld = pb->maps[4 * mi + 3];
        const int64_t rel = t.dst_off - zo;
        if (K <= 0 || t.dst_ld % K) {
            tnk::set_error("plan_tc: stage-2 destination stride is not a whole number of rows");
            return TNK_ERR_ARG;
        }
        tnk_comb_task c = t;
        c.dst_off = off + rel / K * ld + rel % K;
        c.dst_ld = i32(t.dst_ld / K * ld);
        pb->t2.push_back(c);
    }
    // stage 3: A = Z block (m x K), B = R block (n x K)
    for (int64_t i = 0; i < nt3; ++i) {
        const tnk_gemm_task& t = t3[i];
        const int64_t b = (int64_t)pb->s3.size();
        for (int64_t j = t.seg_begin; j < t.seg_end; ++j) {
            const int64_t am = zinfo.at(s3[j].a_off)[2];
            const int64_t bm = staged(KR, s3[j].b_off, t.n, s3[j].k, false);
            pb->s3.push_back(tc_seg(am, bm, s3[j].k));
        }
        pb->t3.push_back(make_task(t.c_off, t.ldc, t.m, t.n, b, (int64_t)pb->s3.size(), 2));
    }
    return TNK_OK;
}

// Stage 3's tasks whose tiles are much longer (in K x tile area) than the average work per
// resident CTA, cut along K into at most max_chunks chunks that write compact partial products
// to the workspace (flags bit 4, from ws_base on), plus the stage-4 combination that sums each
// split task's partials into its output block in chunk order. Output: g3t / g3s (tasks and
// segments), c2t / c2c (stage 4), ws1 = 1 when anything was split, ws2 = workspace added.
int split_build(const tnk_gemm_task* t, int64_t nt, const tnk_gemm_seg* s, int64_t ws_base,
                int slots, int max_chunks, int tile_m, int tile_n, PlanBuild* pb) {
    std::vector<int64_t> ktot(nt), work(nt), chunks(nt);
    int64_t total = 0;
    for (int64_t i = 0; i < nt; ++i) {
        int64_t K = 0;
        for (int64_t j = t[i].seg_begin; j < t[i].seg_end; ++j) K += s[j].k;
        ktot[i] = K;
        work[i] = K * std::min<int64_t>(tile_m, t[i].m) * std::min<int64_t>(tile_n, t[i].n);
        total += work[i] * ((t[i].m + tile_m - 1) / tile_m) * ((t[i].n + tile_n - 1) / tile_n);
    }
    const double target = std::max((double)total / slots, 1.0);
    bool any = false;
    for (int64_t i = 0; i < nt; ++i) {
        chunks[i] = std::min<int64_t>((int64_t)std::ceil((double)work[i] / target), max_chunks);
        any = any || chunks[i] > 1;
    }
    pb->ws1 = any ? 1 : 0;
    if (!any) return TNK_OK;
    int64_t extra = 0;
    for (int64_t i = 0; i < nt; ++i) {
        const tnk_gemm_task& task = t[i];
        const int64_t c = chunks[i];
        if (c <= 1) {
            const int64_t b = (int64_t)pb->g3s.size();
            pb->g3s.insert(pb->g3s.end(), s + task.seg_begin, s + task.seg_end);
            pb->g3t.push_back(make_task(task.c_off, task.ldc, task.m, task.n, b,
                                        (int64_t)pb->g3s.size(), task.flags));
            continue;
        }
        const int64_t m = task.m, n = task.n, K = ktot[i];
        const int64_t tb = (int64_t)pb->c2c.size();
        for (int64_t j = 0; j < c; ++j) {
            const int64_t lo = K * j / c, hi = K * (j + 1) / c;
            const int64_t b = (int64_t)pb->g3s.size();
            int64_t k0 = 0;
            for (int64_t q = task.seg_begin; q < task.seg_end; ++q) {
                const int64_t k = s[q].k;
                const int64_t x0 = std::max(lo, k0), x1 = std::min(hi, k0 + k);
                if (x0 < x1) {
                    tnk_gemm_seg part = s[q];
                    const int64_t d = x0 - k0;
                    part.a_off += d * s[q].a_cs;
                    part.b_off += d * s[q].b_rs;
                    part.k = i32(x1 - x0);
                    pb->g3s.push_back(part);
                }
                k0 += k;
            }
            const int64_t off = ws_base + extra;
            extra += m * n;
            pb->g3t.push_back(make_task(off, n, m, n, b, (int64_t)pb->g3s.size(),
                                        (task.flags & ~1) | 16));
            tnk_comb_term term{};
            term.src_off = off;
            term.src_ld = i32(n);
            term.src_cs = 1;
            term.coef = 1.0;
            pb->c2c.push_back(term);
        }
        tnk_comb_task red{};
        red.dst_off = task.c_off;
        red.rows = i32(m);
        red.cols = i32(n);
        red.dst_ld = task.ldc;
        red.dst_cs = 1;
        red.term_begin = i32(tb);
        red.term_end = i32((int64_t)pb->c2c.size());
        pb->c2t.push_back(red);
    }
    pb->ws2 = extra;
    return TNK_OK;
}

// Environment updates (tnkit/_dmrg.py:216-231) as three stages:
//   left   T[(s,d),(w,q)] = conj(A)[p,(s,d)]^T L[p,(w,q)]          stage 1, per (A, L) block pair
//          U[d, (r, q, y)] = sum_{w,s} W[w,r,s,y] T[(s,d),(w,q)]     stage 2, MPO coefficients
//          L'[(d,r), e] = sum_{q,y} U[(d,r),(q,y)] A[(q,y), e]        stage 3
//   right  T[(u,s),(r,y)] = conj(B)[(u,s),x] R[x,(r,y)]
//          V[u, (w, p, y)] = sum_{r,s} W[w,r,s,p] T[(u,s),(r,y)]
//          R'[(u,w), v] = sum_{p,y} V[(u,w),(p,y)] B[v,(p,y)]^T
// The iteration orders and offsets follow plan.py's plan_left_env / plan_right_env exactly.
int env_build(const tnk_env_plan_in* in, PlanBuild* pb) {
    const bool left = in->side == 0;
    if ((in->side != 0 && in->side != 1) || in->env.nlegs != 3 || in->site.nlegs != 3 ||
        in->out.nlegs != 3 || !in->W || !in->sec_start || !in->sec_dim) {
        tnk::set_error("plan_env: bad arguments");
        return TNK_ERR_ARG;
    }
    const Lay E{&in->env}, S{&in->site}, O{&in->out};
    int64_t st[4];
    st[3] = 1;
    for (int a = 2; a >= 0; --a) st[a] = st[a + 1] * in->w_dims[a + 1];
    auto nsec = [&](int a) { return in->sec_begin[a + 1] - in->sec_begin[a]; };
    auto sstart = [&](int a, int64_t s) { return in->sec_start[in->sec_begin[a] + s]; };
    auto sdim = [&](int a, int64_t s) { return in->sec_dim[in->sec_begin[a] + s]; };
    // W entry at the sectors (w, r, s, t) and offsets (ww, rr, ss, tt) inside them
    auto wval = [&](const int64_t* sec, int64_t ww, int64_t rr, int64_t ss, int64_t tt) {
        return in->W[(sstart(0, sec[0]) + ww) * st[0] + (sstart(1, sec[1]) + rr) * st[1] +
                     (sstart(2, sec[2]) + ss) * st[2] + (sstart(3, sec[3]) + tt) * st[3]];
    };
    auto any_nonzero = [&](const int64_t* sec) {
        for (int a = 0; a < 4; ++a)
            if (sec[a] < 0 || sec[a] >= nsec(a)) throw std::out_of_range("MPO sector");
        for (int64_t a = 0; a < sdim(0, sec[0]); ++a)
            for (int64_t b = 0; b < sdim(1, sec[1]); ++b)
                for (int64_t c = 0; c < sdim(2, sec[2]); ++c)
                    for (int64_t d = 0; d < sdim(3, sec[3]); ++d)
                        if (wval(sec, a, b, c, d) != 0.0) return true;
        return false;
    };
    using TK = std::array<int64_t, 4>;
    std::unordered_map<int64_t, std::vector<int64_t>> env_by0, site_by;
    for (int64_t k = 0; k < E.nb(); ++k) env_by0[E.key(k, 0)].push_back(k);
    for (int64_t k = 0; k < S.nb(); ++k) site_by[S.key(k, left ? 2 : 0)].push_back(k);
    std::map<TK, std::pair<int64_t, int64_t>> tcand;
    std::map<std::pair<int64_t, int64_t>, std::vector<TK>> t_by;
    for (int64_t ks = 0; ks < S.nb(); ++ks) {
        const int64_t s0 = S.key(ks, 0), s1 = S.key(ks, 1), s2 = S.key(ks, 2);
        auto it = env_by0.find(left ? s0 : s2);
        if (it == env_by0.end()) continue;
        for (int64_t ke : it->second) {
            const int64_t e1 = E.key(ke, 1), e2 = E.key(ke, 2);
            // left: (s, d, w, q); right: (u, s, r, y)
            const TK tk = left ? TK{s1, s2, e1, e2} : TK{s0, s1, e1, e2};
            tcand[tk] = {ks, ke};
            t_by[left ? std::make_pair(s2, e2) : std::make_pair(s0, e2)].push_back(tk);
        }
    }
    struct Contrib {
        TK tk;
        int64_t sec[4];
    };
    struct Def {
        int64_t a, b, c, d, ks2;     // left: D, Rd, Q, Yd; right: U, Wd, Pd, Yd
        std::vector<Contrib> contrib;
    };
    std::vector<Def> defs;
    std::vector<std::pair<int64_t, std::vector<int64_t>>> tasks3;
    for (int64_t ko = 0; ko < O.nb(); ++ko) {
        const int64_t o0 = O.key(ko, 0), o1 = O.key(ko, 1), o2 = O.key(ko, 2);
        std::vector<int64_t> segs3;
        auto sit = site_by.find(left ? o2 : o2);
        if (sit != site_by.end()) {
            for (int64_t ks2 : sit->second) {
                Def df{};
                df.ks2 = ks2;
                const int64_t k0 = S.key(ks2, 0), k1 = S.key(ks2, 1);
                auto tit = t_by.find({o0, left ? k0 : S.key(ks2, 2)});
                if (tit != t_by.end()) {
                    for (const TK& tk : tit->second) {
                        Contrib cb{};
                        cb.tk = tk;
                        if (left) {   // W[w, r, s, y]: w = tk[2], r = o1, s = tk[0], y = k1
                            cb.sec[0] = tk[2]; cb.sec[1] = o1; cb.sec[2] = tk[0]; cb.sec[3] = k1;
                        } else {      // W[w, r, s, p]: w = o1, r = tk[2], s = tk[1], p = k1
                            cb.sec[0] = o1; cb.sec[1] = tk[2]; cb.sec[2] = tk[1]; cb.sec[3] = k1;
                        }
                        if (any_nonzero(cb.sec)) df.contrib.push_back(cb);
                    }
                }
                if (df.contrib.empty()) continue;
                if (left) {
                    df.a = O.shape(ko, 0); df.b = O.shape(ko, 1);
                    df.c = S.shape(ks2, 0); df.d = S.shape(ks2, 1);
                } else {
                    df.a = O.shape(ko, 0); df.b = O.shape(ko, 1);
                    df.c = S.shape(ks2, 1); df.d = S.shape(ks2, 2);
                }
                defs.push_back(std::move(df));
                segs3.push_back((int64_t)defs.size() - 1);
            }
        }
        tasks3.emplace_back(ko, std::move(segs3));
    }
    // stage 1: the T blocks some U / V block uses, in order of first use
    std::map<TK, int64_t> t_off;
    for (const Def& df : defs)
        for (const Contrib& cb : df.contrib) {
            if (t_off.count(cb.tk)) continue;
            const auto [ks, ke] = tcand.at(cb.tk);
            const int64_t b = (int64_t)pb->g1s.size();
            t_off[cb.tk] = pb->ws1;
            int64_t m, n, k;
            if (left) {   // A (P, S, D) x L (P, Wd, Q)
                const int64_t P = S.shape(ks, 0), Sd = S.shape(ks, 1), D = S.shape(ks, 2);
                const int64_t Wd = E.shape(ke, 1), Q = E.shape(ke, 2);
                m = Sd * D; n = Wd * Q; k = P;
                pb->g1s.push_back(make_seg(S.off(ks), 1, Sd * D, SLOT_X0, E.off(ke), Wd * Q, 1,
                                           SLOT_X1, P));
            } else {      // B (U, S, X) x R (X, Rd, Yd)
                const int64_t U = S.shape(ks, 0), Sd = S.shape(ks, 1), X = S.shape(ks, 2);
                const int64_t Rd = E.shape(ke, 1), Yd = E.shape(ke, 2);
                m = U * Sd; n = Rd * Yd; k = X;
                pb->g1s.push_back(make_seg(S.off(ks), X, 1, SLOT_X0, E.off(ke), Rd * Yd, 1,
                                           SLOT_X1, X));
            }
            pb->g1s.back().conj = 1;
            pb->g1t.push_back(make_task(pb->ws1, n, m, n, b, b + 1, 0));
            pb->macs1 += m * n * k;
            pb->ws1 += m * n;
        }
    // stage 2
    std::vector<int64_t> d_off;
    for (const Def& df : defs) {
        const int64_t base = pb->ws1 + pb->ws2;
        d_off.push_back(base);
        pb->ws2 += df.a * df.b * df.c * df.d;
        if (left) {   // rows D, cols Q, for each (rr, yy)
            const int64_t D = df.a, Rd = df.b, Q = df.c, Yd = df.d;
            for (int64_t rr = 0; rr < Rd; ++rr)
                for (int64_t yy = 0; yy < Yd; ++yy) {
                    const int64_t tb = (int64_t)pb->c2c.size();
                    for (const Contrib& cb : df.contrib) {
                        const auto [ks, ke] = tcand.at(cb.tk);
                        const int64_t Sd = S.shape(ks, 1), Dd = S.shape(ks, 2);
                        const int64_t Wd = E.shape(ke, 1), Qd = E.shape(ke, 2);
                        for (int64_t ww = 0; ww < Wd; ++ww)
                            for (int64_t ss = 0; ss < Sd; ++ss) {
                                const double c = wval(cb.sec, ww, rr, ss, yy);
                                if (c == 0.0) continue;
                                tnk_comb_term t{};
                                t.src_off = t_off.at(cb.tk) + ss * Dd * Wd * Qd + ww * Qd;
                                t.src_ld = i32(Wd * Qd);
                                t.src_cs = 1;
                                t.coef = c;
                                pb->c2c.push_back(t);
                            }
                    }
                    tnk_comb_task c{};
                    c.dst_off = base + rr * Q * Yd + yy;
                    c.rows = i32(D);
                    c.cols = i32(Q);
                    c.dst_ld = i32(Rd * Q * Yd);
                    c.dst_cs = i32(Yd);
                    c.term_begin = i32(tb);
                    c.term_end = i32((int64_t)pb->c2c.size());
                    pb->c2t.push_back(c);
                }
        } else {      // rows U, cols Yd, for each (ww, pp)
            const int64_t U = df.a, Wd = df.b, Pd = df.c, Yd = df.d;
            for (int64_t ww = 0; ww < Wd; ++ww)
                for (int64_t pp = 0; pp < Pd; ++pp) {
                    const int64_t tb = (int64_t)pb->c2c.size();
                    for (const Contrib& cb : df.contrib) {
                        const auto [ks, ke] = tcand.at(cb.tk);
                        const int64_t Sd = S.shape(ks, 1), Rd = E.shape(ke, 1);
                        for (int64_t ss = 0; ss < Sd; ++ss)
                            for (int64_t rr = 0; rr < Rd; ++rr) {
                                const double c = wval(cb.sec, ww, rr, ss, pp);
                                if (c == 0.0) continue;
                                tnk_comb_term t{};
                                t.src_off = t_off.at(cb.tk) + (ss * Rd + rr) * Yd;
                                t.src_ld = i32(Sd * Rd * Yd);
                                t.src_cs = 1;
                                t.coef = c;
                                pb->c2c.push_back(t);
                            }
                    }
                    tnk_comb_task c{};
                    c.dst_off = base + (ww * Pd + pp) * Yd;
                    c.rows = i32(U);
                    c.cols = i32(Yd);
                    c.dst_ld = i32(Wd * Pd * Yd);
                    c.dst_cs = 1;
                    c.term_begin = i32(tb);
                    c.term_end = i32((int64_t)pb->c2c.size());
                    pb->c2t.push_back(c);
                }
        }
    }
    // stage 3
    for (const auto& [ko, segs3] : tasks3) {
        const int64_t b = (int64_t)pb->g3s.size();
        const int64_t o0 = O.shape(ko, 0), o1 = O.shape(ko, 1), o2 = O.shape(ko, 2);
        for (int64_t di : segs3) {
            const Def& df = defs[di];
            const int64_t K = df.c * df.d;
            if (left)
                pb->g3s.push_back(make_seg(d_off[di], K, 1, SLOT_WS, S.off(df.ks2), o2, 1,
                                           SLOT_X2, K));
            else
                pb->g3s.push_back(make_seg(d_off[di], K, 1, SLOT_WS, S.off(df.ks2), 1, K,
                                           SLOT_X2, K));
            pb->macs3 += o0 * o1 * o2 * K;
        }
        pb->g3t.push_back(make_task(O.off(ko), o2, o0 * o1, o2, b, (int64_t)pb->g3s.size(), 0));
    }
    return TNK_OK;
}

// Block tensordot (tnkit/blocks.py:1156-1192): out = a . b over the last nc legs of a and the
// first nc legs of b; one GEMM task per output block with one K segment per matching (a, b)
// block pair, in plan.py's plan_tensordot order.
int tensordot_build(const tnk_layout_desc* ad, const tnk_layout_desc* bd,
                    const tnk_layout_desc* od, int nc, PlanBuild* pb) {
    const Lay a{ad}, b{bd}, o{od};
    const int na = ad->nlegs, nb = bd->nlegs;
    if (nc < 0 || nc > na || nc > nb || od->nlegs != na + nb - 2 * nc) {
        tnk::set_error("plan_tensordot: bad leg counts");
        return TNK_ERR_ARG;
    }
    using Key = std::vector<int64_t>;
    auto key = [](const Lay& t, int64_t k, int l0, int l1) {
        Key v;
        for (int l = l0; l < l1; ++l) v.push_back(t.key(k, l));
        return v;
    };
    std::map<Key, std::vector<int64_t>> b_by_k, a_by_free;
    for (int64_t k = 0; k < b.nb(); ++k) b_by_k[key(b, k, 0, nc)].push_back(k);
    for (int64_t k = 0; k < a.nb(); ++k) a_by_free[key(a, k, 0, na - nc)].push_back(k);
    for (int64_t ko = 0; ko < o.nb(); ++ko) {
        const Key fa = key(o, ko, 0, na - nc), fb = key(o, ko, na - nc, od->nlegs);
        int64_t M = 1, N = 1;
        for (int l = 0; l < na - nc; ++l) M *= o.shape(ko, l);
        for (int l = na - nc; l < od->nlegs; ++l) N *= o.shape(ko, l);
        const int64_t s0 = (int64_t)pb->g1s.size();
        auto ait = a_by_free.find(fa);
        if (ait != a_by_free.end()) {
            for (int64_t ka : ait->second) {
                auto bit = b_by_k.find(key(a, ka, na - nc, na));
                if (bit == b_by_k.end()) continue;
                for (int64_t kb : bit->second) {
                    if (key(b, kb, nc, nb) != fb) continue;
                    int64_t K = 1;
                    for (int l = na - nc; l < na; ++l) K *= a.shape(ka, l);
                    pb->g1s.push_back(make_seg(a.off(ka), K, 1, SLOT_X0, b.off(kb), N, 1,
                                               SLOT_X1, K));
                    pb->macs1 += M * N * K;
                }
            }
        }
        pb->g1t.push_back(make_task(o.off(ko), N, M, N, s0, (int64_t)pb->g1s.size(), 0));
    }
    return TNK_OK;
}

template <typename T>
void table(const std::vector<T>& v, const void** data, int64_t* count) {
    *data = v.empty() ? nullptr : (const void*)v.data();
    *count = (int64_t)v.size();
}

// Runs one builder into a fresh PlanBuild with every C++ exception turned into a status code
// (no exception may cross the C ABI: a ctypes caller would abort), then hands the plan over.
template <typename F>
int guarded_build(const char* what, void** handle, F&& build) {
    PlanBuild* pb = nullptr;
    int rc;
    try {
        pb = new PlanBuild();
        rc = build(pb);
    } catch (const Overflow&) {
        tnk::set_error("%s: a table entry exceeds 32 bits", what);
        rc = TNK_ERR_SIZE;
    } catch (const std::bad_alloc&) {
        tnk::set_error("%s: out of host memory", what);
        rc = TNK_ERR_SIZE;
    } catch (const std::exception& e) {
        tnk::set_error("%s: %s", what, e.what());
        rc = TNK_ERR_ARG;
    } catch (...) {
        tnk::set_error("%s: unexpected exception", what);
        rc = TNK_ERR_ARG;
    }
    if (rc) {
        delete pb;
        return rc;
    }
    *handle = pb;
    return TNK_OK;
}

}  // namespace

extern "C" int tnk_apply_plan_build(const tnk_apply_plan_in* in, void** handle) {
    if (!in || !handle) {
        tnk::set_error("tnk_apply_plan_build: null argument");
        return TNK_ERR_ARG;
    }
    *handle = nullptr;
    return guarded_build("plan_apply", handle,
                         [&](PlanBuild* pb) { return apply_build(in, pb); });
}

extern "C" int tnk_env_plan_build(const tnk_env_plan_in* in, void** handle) {
    if (!in || !handle) {
        tnk::set_error("tnk_env_plan_build: null argument");
        return TNK_ERR_ARG;
    }
    *handle = nullptr;
    return guarded_build("plan_env", handle,
                         [&](PlanBuild* pb) { return env_build(in, pb); });
}

extern "C" int tnk_tensordot_plan_build(const tnk_layout_desc* a, const tnk_layout_desc* b,
                                        const tnk_layout_desc* out, int32_t nc,
                                        void** handle) {
    if (!a || !b || !out || !handle) {
        tnk::set_error("tnk_tensordot_plan_build: null argument");
        return TNK_ERR_ARG;
    }
    *handle = nullptr;
    return guarded_build("plan_tensordot", handle,
                         [&](PlanBuild* pb) { return tensordot_build(a, b, out, nc, pb); });
}

extern "C" int tnk_plan_tc_build(const tnk_gemm_task* t1, int64_t nt1, const tnk_gemm_seg* s1,
                                 const tnk_comb_task* t2, int64_t nt2, const tnk_gemm_task* t3,
                                 int64_t nt3, const tnk_gemm_seg* s3, void** handle) {
    if (!handle || nt1 < 0 || nt2 < 0 || nt3 < 0 || (nt1 && (!t1 || !s1)) || (nt2 && !t2) ||
        (nt3 && (!t3 || !s3))) {
        tnk::set_error("tnk_plan_tc_build: bad argument");
        return TNK_ERR_ARG;
    }
    *handle = nullptr;
    return guarded_build("plan_tc", handle,
                         [&](PlanBuild* pb) { return tc_build(t1, nt1, s1, t2, nt2, t3, nt3, s3, pb); });
}

extern "C" int tnk_plan_split_k(const tnk_gemm_task* t, int64_t nt, const tnk_gemm_seg* s,
                                int64_t ws_base, int32_t slots, int32_t max_chunks,
                                int32_t tile_m, int32_t tile_n, void** handle) {
    if (!handle || nt < 0 || (nt && (!t || !s)) || slots < 1 || max_chunks < 1 || tile_m < 1 ||
        tile_n < 1) {
        tnk::set_error("tnk_plan_split_k: bad argument");
        return TNK_ERR_ARG;
    }
    *handle = nullptr;
    return guarded_build("plan_split_k", handle,
                         [&](PlanBuild* pb) { return split_build(t, nt, s, ws_base, slots, max_chunks, tile_m, tile_n, pb); });
}

extern "C" int tnk_planb_table(const void* handle, int32_t id, const void** data,
                               int64_t* count) {
    if (!handle || !data || !count) {
        tnk::set_error("tnk_planb_table: null argument");
        return TNK_ERR_ARG;
    }
    const PlanBuild* pb = static_cast<const PlanBuild*>(handle);
    switch (id) {
        case 0: table(pb->g1t, data, count); break;
        case 1: table(pb->g1s, data, count); break;
        case 2: table(pb->c2t, data, count); break;
        case 3: table(pb->c2c, data, count); break;
        case 4: table(pb->g3t, data, count); break;
        case 5: table(pb->g3s, data, count); break;
        case 10: table(pb->t1, data, count); break;
        case 11: table(pb->s1, data, count); break;
        case 12: table(pb->t2, data, count); break;
        case 13: table(pb->t3, data, count); break;
        case 14: table(pb->s3, data, count); break;
        case 15:
            *data = pb->maps.empty() ? nullptr : (const void*)pb->maps.data();
            *count = (int64_t)pb->maps.size() / 4;
            break;
        case 16: case 17: case 18: table(pb->cvt[id - 16], data, count); break;
        default:
            tnk::set_error("tnk_planb_table: unknown table %d", id);
            return TNK_ERR_ARG;
    }
    return TNK_OK;
}

extern "C" int tnk_planb_scalars(const void* handle, int64_t* out5) {
    if (!handle || !out5) {
        tnk::set_error("tnk_planb_scalars: null argument");
        return TNK_ERR_ARG;
    }
    const PlanBuild* pb = static_cast<const PlanBuild*>(handle);
    out5[0] = pb->ws1;
    out5[1] = pb->ws2;
    out5[2] = pb->macs1;
    out5[3] = pb->macs3;
    out5[4] = pb->cursor;
    return TNK_OK;
}

extern "C" void tnk_planb_free(void* handle) { delete static_cast<PlanBuild*>(handle); }
