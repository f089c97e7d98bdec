"""A numpy interpreter of the kernel task tables (include/tnkit_gb300.h semantics).

Test helper only: it lets the CPU suite check that the host planners emit correct tables
(against the oracle and the reference's golden vectors) without a GPU. The product never runs it.
"""
import numpy as np
from numpy.lib.stride_tricks import as_strided


def _view(buf, off, shape, strides):
    it = buf.itemsize
    return as_strided(buf[int(off):], shape=tuple(int(s) for s in shape),
                      strides=tuple(int(s) * it for s in strides), writeable=False)


def run_gemm(tables, slots, C):
    tasks, segs, tiles = tables
    covered = np.zeros(len(tasks), bool)
    for t in tiles:
        covered[t["task"]] = True
    for ti, t in enumerate(tasks):
        m, n = int(t["m"]), int(t["n"])
        assert covered[ti] or m == 0 or n == 0, "task without tiles"
        acc = np.zeros((m, n))
        for s in segs[int(t["seg_begin"]):int(t["seg_end"])]:
            k = int(s["k"])
            A = _view(slots[int(s["a_buf"])], s["a_off"], (m, k), (s["a_rs"], s["a_cs"]))
            B = _view(slots[int(s["b_buf"])], s["b_off"], (k, n), (s["b_rs"], s["b_cs"]))
            acc += float(s["coef"]) * (A @ B)
        ccs = 2 if int(t["flags"]) & 4 else 1
        idx = (int(t["c_off"]) + np.arange(m)[:, None] * int(t["ldc"])
               + np.arange(n)[None, :] * ccs)
        dst = slots[3] if int(t["flags"]) & 16 else C
        if int(t["flags"]) & 1:
            dst[idx] += acc
        else:
            dst[idx] = acc


def run_comb(tables, src, dst):
    tasks, terms, items = tables
    for t in tasks:
        rows, cols = int(t["rows"]), int(t["cols"])
        acc = np.zeros((rows, cols))
        for u in terms[int(t["term_begin"]):int(t["term_end"])]:
            acc += float(u["coef"]) * _view(src, u["src_off"], (rows, cols),
                                            (u["src_ld"], u["src_cs"]))
        idx = (int(t["dst_off"]) + np.arange(rows)[:, None] * int(t["dst_ld"])
               + np.arange(cols)[None, :] * int(t["dst_cs"]))
        dst[idx] = acc
    # every row of every task is in exactly one item
    seen = {}
    for it in items:
        seen.setdefault(int(it["task"]), []).append((int(it["row0"]), int(it["row1"])))
    for ti, t in enumerate(tasks):
        rs = sorted(seen.get(ti, []))
        if int(t["rows"]) and int(t["cols"]):
            assert rs[0][0] == 0 and rs[-1][1] == int(t["rows"])
            assert all(a[1] == b[0] for a, b in zip(rs, rs[1:]))


def run_plan3(plan, x0, x1, x2):
    ws = np.zeros(plan.ws1 + plan.ws2)
    scale = 2 if getattr(plan, "kind", "").endswith("c128") else 1
    out = np.zeros(plan.out_layout.size * scale)
    slots = [x0, x1, x2, ws]
    run_gemm(plan.g1, slots, ws)
    run_comb(plan.c2, ws.copy(), ws)
    run_gemm(plan.g3, slots, out)
    c4 = getattr(plan, "c4", None)
    if c4 is not None and len(c4[0]):
        run_comb(c4, ws, out)
    return out


def tf32(x):
    """Round float32 values to TF32 (10 explicit mantissa bits, nearest, ties away from zero)."""
    u = np.asarray(x, np.float32).view(np.uint32)
    return ((u + np.uint32(0x1000)) & np.uint32(0xFFFFE000)).view(np.float32)


def run_tc_plan(tc, L, theta, R, passes=3):
    """Interpret a HostPlanTC: staging, two split-TF32 GEMM stages over tensor-map blocks, the
    FP32 combination, FP64 output."""
    S = tc.stage_elems
    stage = np.full(2 * S, np.nan, np.float32)

    def cvt(tasks, src):
        for t in tasks:
            rows, cols = int(t["rows"]), int(t["cols"])
            blk = _view(src, t["src_off"], (rows, cols), (t["src_ld"], 1))
            if int(t["transpose"]):
                blk = blk.T
            x = np.asarray(blk, np.float64)
            h = tf32(x.astype(np.float32)) if passes == 3 else x.astype(np.float32)
            lo = tf32((x - h.astype(np.float64)).astype(np.float32))
            r, c = h.shape
            idx = int(t["dst_off"]) + np.arange(r)[:, None] * int(t["dst_ld"]) + np.arange(c)[None, :]
            stage[idx] = h
            stage[S + idx] = lo
    cvt(tc.cvt["L"], L)
    cvt(tc.cvt["R"], R)
    cvt(tc.cvt["T"], theta)

    def block(mi, lo=False):
        off, r, c, ld = tc.maps[mi]
        base = S if lo else 0
        idx = base + off + np.arange(r)[:, None] * ld + np.arange(c)[None, :]
        return stage[idx].astype(np.float32)

    def gemm(tasks, segs, out, f64):
        for t in tasks:
            m, n = int(t["m"]), int(t["n"])
            acc = np.zeros((m, n), np.float32)
            for s in segs[int(t["seg_begin"]):int(t["seg_end"])]:
                Ah, Bh = block(int(s["a_map"])), block(int(s["b_map"]))
                assert Ah.shape[0] == m and Bh.shape[0] == n and Ah.shape[1] == Bh.shape[1] == int(s["k"])
                acc += Ah @ Bh.T
                if passes == 3:
                    acc += Ah @ block(int(s["b_map"]), True).T + block(int(s["a_map"]), True) @ Bh.T
            idx = int(t["c_off"]) + np.arange(m)[:, None] * int(t["ldc"]) + np.arange(n)[None, :]
            out[idx] = acc.astype(out.dtype)
    y32 = np.zeros(tc.y32_elems, np.float32)
    gemm(tc.t1, tc.s1, y32, False)
    for t in tc.t2:
        rows, cols = int(t["rows"]), int(t["cols"])
        acc = np.zeros((rows, cols), np.float32)
        for u in tc.c2[int(t["term_begin"]):int(t["term_end"])]:
            acc += np.float32(u["coef"]) * _view(y32, u["src_off"], (rows, cols), (u["src_ld"], u["src_cs"]))
        idx = int(t["dst_off"]) + np.arange(rows)[:, None] * int(t["dst_ld"]) + np.arange(cols)[None, :] * int(t["dst_cs"])
        h = tf32(acc) if passes == 3 else acc
        stage[idx] = h
        stage[S + idx] = tf32(acc - h)
    out = np.zeros(tc.out_layout.size)
    gemm(tc.t3, tc.s3, out, True)
    return out
