"""Generate the golden fixtures of this directory by running the reference tnkit itself.

This script is test infrastructure. It imports the reference package read-only from the
checkout given by ``--ref`` (or the ``TNKIT_REF`` environment variable; one of the two is
required) and writes small JSON / NPZ fixtures next to itself. The fixtures are committed; the
script is not needed at test time.

usage:
  export TNKIT_REF=<path of a tnkit 0.3.0 checkout>
  PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py small      # seconds
  PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py dmrg       # a few minutes
  PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py c2         # ~30 min on 8 cores
  PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py hubbard    # a minute

Modes:
  small  Block and dense local problems (L, W1, W2, R, theta) dumped from real reference DMRG
         runs at small sizes, with the reference's own outputs of apply_two_site,
         apply_one_site, update_left_env, update_right_env and truncated_svd, plus a thick-restart
         Lanczos known answer.  -> local_problems.npz, local_problems.json
  dmrg   Per-sweep energies of whole reference DMRG runs at small and medium sizes (TFIM N=10
         chi=32 dense; XXZ N=12 U(1); XXZ N=64 U(1) at chi=64/128), with the discarded weight
         and every bond's entanglement entropy of the final state (the reference's
         all_entropies of its to_dense_mps).  -> dmrg_small.json
  c2     The XXZ N=64 U(1) chi=1024 six-sweep run: energies, sweep times, matvec counts, every
         bond's sector dims, every bond's entropy and the mid bond's Schmidt spectrum.
         -> c2_xxz_n64_chi1024.json
  hubbard  The Fermi-Hubbard chain (t=1, U=4, half filling) under U(1) x U(1) (N_up, N_dn)
         blocks, with the hand-written width-6 MPO of tnkit_gb300/workloads.py: the
         reference's block MPO tensor of a bulk site, its seeded random block MPS, and the
         per-sweep energies of its block DMRG (N=6 chi=16, N=8 chi=32), with the exact ground
         energy of N=6 from the dense Hamiltonian.  -> hubbard_u1u1.npz, hubbard_u1u1.json
  grad   Hellmann-Feynman coupling gradients of the disordered XXZ chain (N=10, J_i uniform in
         [0.5, 1.5] from seed 2, delta=1) on complex U(1) blocks: the reference's ground state
         and, per bond, its mpo_expectation of dH/dJ_i (the one-bond MPO), with central finite
         differences of the reference's energies (h=1e-5) at three bonds.  -> grad_xxz10.json
  tdvp   Two-site TDVP of the XXZ N=10 chain on complex U(1) blocks from a seeded random state:
         the initial tensors, the reference's Krylov exponential on a fixed vector, and the
         state vector after 4 steps of dt=0.05.  -> tdvp_xxz10.npz, tdvp_xxz10.json
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _import_ref(path):
    sys.dont_write_bytecode = True
    sys.path.insert(0, path)
    import tnkit  # noqa: F401
    return tnkit


def xxz_bulk(delta=1.0):
    """Bulk MPO of H = sum (S+S- + S-S+)/2 + delta SzSz (spin 1/2), channels (idle, S+, S-, Sz,
    done): the MPO of the reference's bench/profile/fused_dmrg_check.py:48-53 at delta = 1."""
    sp = np.array([[0.0, 1.0], [0.0, 0.0]])
    sm = sp.T.copy()
    sz = np.diag([0.5, -0.5])
    i2 = np.eye(2)
    W = np.zeros((5, 5, 2, 2))
    W[0, 0], W[0, 1], W[0, 2], W[0, 3] = i2, sp, sm, sz
    W[1, 4], W[2, 4], W[3, 4], W[4, 4] = 0.5 * sm, 0.5 * sp, delta * sz, i2
    return W


def open_chain(Wb, N):
    D = Wb.shape[0]
    return [Wb[0:1] if i == 0 else Wb[:, D - 1:D] if i == N - 1 else Wb for i in range(N)]


def _legs_json(struct):
    return [{"charges": [int(c) for c in leg.charges], "dims": [int(d) for d in leg.dims],
             "sign": int(leg.sign)} for leg in struct.legs]


def _bt(prefix, t, arrays, meta):
    """Record a reference BlockTensor: canonical buffer into `arrays`, legs/charge into `meta`."""
    t = t.canonical()
    arrays[prefix] = np.asarray(t.data)
    meta[prefix] = {"legs": _legs_json(t.struct), "charge": int(t.struct.charge)}


def _block_spectra(mps, site_charges):
    """Every bond's entropy of a block MPS and its Schmidt spectra, by the reference's own
    route: to_dense_mps (tnkit/block_backend.py:462-466), then the one-sweep
    _schmidt_sweep / _entropy of all_entropies (tnkit/observables.py:313-387)."""
    from tnkit.block_backend import to_dense_mps
    from tnkit.observables import _canon, _entropy, _schmidt_sweep, _backend_for
    dense = [np.asarray(t) for t in to_dense_mps(mps, site_charges)]
    be = _backend_for(dense)
    canon = _canon(dense, be)
    spectra = [np.asarray(s, dtype=np.float64) for s in _schmidt_sweep(canon, be, len(dense) - 1)]
    return [float(_entropy(s)) for s in spectra], spectra


def mode_small(ref):
    from tnkit import dmrg, get_backend, U1, to_block_mpo
    from tnkit import _dmrg as D
    from tnkit.blocks import truncated_svd
    from tnkit.legs import fuse
    from tnkit.eigensolver import lanczos_ground_restart
    from tnkit.models import tfim_mpo

    arrays, meta = {}, {}
    be = get_backend("numpy-real")
    # --- U(1) XXZ N=12 chi=16: a converged state, local problem at bonds 5 (mid) and 0 (edge)
    N = 12
    W = open_chain(xxz_bulk(1.0), N)
    Wb, _ = to_block_mpo(W, [[1, -1]] * N, be, sym=U1())
    E, mps, info = dmrg(Wb, 16, charge=0, seed=1, n_sweeps=4, tol=0, rtol=0, expand=0,
                        backend="numpy-real")
    meta["xxz12"] = {"E": float(E), "energies": [float(e) for e in info["energies"]]}
    bbe = D._block_backend("numpy-real", Wb, None)
    M = list(mps)
    Wd = [bbe.array(w) for w in Wb]
    Ls = [None] * (N + 1)
    Rs = [None] * (N + 1)
    Ls[0], Rs[N] = D._edge_envs(M, Wd, bbe)
    for i in range(N - 1, 0, -1):
        Rs[i] = D.update_right_env(Rs[i + 1], M[i], Wd[i], bbe)
    # move the centre right to bond `mid` with QR-free SVD splits in the reference itself
    rng = np.random.default_rng(7)
    for i in range(N - 1):
        Ls[i + 1] = None
    for bond in (0, 5):
        # left envs up to `bond`: left-canonicalise by truncated_svd of the reference
        M = list(mps)
        Lc = Ls[0]
        for i in range(bond):
            th = bbe.einsum("asc,ctb->astb", M[i], M[i + 1])
            mat, rec = fuse(th, ((0, 1), (2, 3)), bbe)
            U, S, Vh, _ = truncated_svd(mat, 10 ** 6)
            from tnkit.legs import split
            M[i] = split(U, rec, bbe, legs=(0,))
            M[i + 1] = split(Vh.scale(S, 0), rec, bbe, legs=(1,))
            Lc = D.update_left_env(Lc, M[i], Wd[i], bbe)
        th = bbe.einsum("asc,ctb->astb", M[bond], M[bond + 1])
        # a random theta with the same layout makes the matvec test independent of the state
        rnd = th.canonical()
        rnd = type(rnd)(rnd.struct, rng.standard_normal(rnd.struct.size))
        tag = f"xxz12_b{bond}"
        _bt(f"{tag}_L", Lc, arrays, meta)
        _bt(f"{tag}_R", Rs[bond + 2], arrays, meta)
        _bt(f"{tag}_W1", Wd[bond], arrays, meta)
        _bt(f"{tag}_W2", Wd[bond + 1], arrays, meta)
        _bt(f"{tag}_theta", rnd, arrays, meta)
        _bt(f"{tag}_H2theta", D.apply_two_site(rnd, Lc, Wd[bond], Wd[bond + 1], Rs[bond + 2],
                                               bbe), arrays, meta)
        # one-site matvec and environment growth on the left site tensor A = M[bond]
        A = M[bond].canonical()
        Ar = type(A)(A.struct, rng.standard_normal(A.struct.size))
        _bt(f"{tag}_A", Ar, arrays, meta)
        _bt(f"{tag}_R1", Rs[bond + 1], arrays, meta)
        _bt(f"{tag}_H1A", D.apply_one_site(Ar, Lc, Wd[bond], Rs[bond + 1], bbe), arrays, meta)
        _bt(f"{tag}_Lnext", D.update_left_env(Lc, Ar, Wd[bond], bbe), arrays, meta)
        B = M[bond + 1].canonical()
        Br = type(B)(B.struct, rng.standard_normal(B.struct.size))
        _bt(f"{tag}_B", Br, arrays, meta)
        _bt(f"{tag}_Rnext", D.update_right_env(Rs[bond + 2], Br, Wd[bond + 1], bbe), arrays,
            meta)
        # truncated SVD of the (real, converged) two-site block
        mat, rec = fuse(th, ((0, 1), (2, 3)), bbe)
        for chi in (4, 10 ** 6):
            U, S, Vh, disc = truncated_svd(mat, chi)
            _bt(f"{tag}_svdin", mat, arrays, meta)
            arrays[f"{tag}_S_chi{chi}"] = np.asarray(S)
            meta[f"{tag}_S_chi{chi}"] = {"disc": float(disc),
                                         "bond": _legs_json(U.struct)[1]}
    # --- dense TFIM N=10: local problem at bond 4 from a converged chi=32 state
    Wt = [np.real(w) for w in tfim_mpo(10, 1.0)]
    E, mps, info = dmrg(Wt, 32, n_sweeps=10, tol=0, rtol=0, seed=0, backend="numpy-real")
    meta["tfim10"] = {"E": float(E), "energies": [float(e) for e in info["energies"]]}
    M = list(mps)
    Ls = [np.ones((1, 1, 1))]
    Rs = [None] * 11
    Rs[10] = np.ones((1, 1, 1))
    for i in range(9, 0, -1):
        Rs[i] = D.update_right_env(Rs[i + 1], M[i], Wt[i], be)
    rng = np.random.default_rng(11)
    L0 = np.ones((1, 1, 1))
    Lc = L0
    for i in range(4):
        th = np.einsum("asc,ctb->astb", M[i], M[i + 1])
        a, s, t, b = th.shape
        U, S, Vh = np.linalg.svd(th.reshape(a * s, t * b), full_matrices=False)
        k = min(32, len(S))
        M[i] = U[:, :k].reshape(a, s, k)
        M[i + 1] = (S[:k, None] * Vh[:k]).reshape(k, t, b)
        Lc = D.update_left_env(Lc, M[i], Wt[i], be)
    th = rng.standard_normal(np.einsum("asc,ctb->astb", M[4], M[5]).shape)
    arrays["tfim10_b4_L"] = Lc
    arrays["tfim10_b4_R"] = Rs[6]
    arrays["tfim10_b4_W1"] = Wt[4]
    arrays["tfim10_b4_W2"] = Wt[5]
    arrays["tfim10_b4_theta"] = th
    arrays["tfim10_b4_H2theta"] = D.apply_two_site(th, Lc, Wt[4], Wt[5], Rs[6], be)
    A = rng.standard_normal(M[4].shape)
    arrays["tfim10_b4_A"] = A
    arrays["tfim10_b4_Lnext"] = D.update_left_env(Lc, A, Wt[4], be)
    B = rng.standard_normal(M[5].shape)
    arrays["tfim10_b4_B"] = B
    arrays["tfim10_b4_Rnext"] = D.update_right_env(Rs[6], B, Wt[5], be)
    # --- thick-restart Lanczos known answer on a fixed symmetric matrix (restarts exercised)
    rng = np.random.default_rng(3)
    n = 300
    Q = rng.standard_normal((n, n))
    Hs = 0.5 * (Q + Q.T) + np.diag(np.linspace(-3.0, 3.0, n))
    v0 = rng.standard_normal(n)
    e, x, linfo = lanczos_ground_restart(lambda v: Hs @ v, v0, be, tol=1e-10, max_iter=400,
                                         m=20, k=5)
    arrays["lanczos_H"] = Hs
    arrays["lanczos_v0"] = v0
    arrays["lanczos_x"] = np.asarray(x)
    meta["lanczos"] = {"e": float(e), "iters": int(linfo["iters"]),
                       "restarts": int(linfo["restarts"]), "m": 20, "k": 5, "tol": 1e-10,
                       "max_iter": 400, "eigvalsh0": float(np.linalg.eigvalsh(Hs)[0])}
    np.savez_compressed(os.path.join(HERE, "local_problems.npz"), **arrays)
    with open(os.path.join(HERE, "local_problems.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print("wrote local_problems.{npz,json}:", len(arrays), "arrays")


def mode_dmrg(ref):
    from tnkit import dmrg, get_backend, U1, to_block_mpo
    from tnkit.models import tfim_mpo
    from tnkit.free_fermion import tfim_free_fermion_energy
    out = {}
    Wt = [np.real(w) for w in tfim_mpo(10, 1.0)]
    t0 = time.perf_counter()
    E, mps, info = dmrg(Wt, 32, n_sweeps=10, tol=0, rtol=0, seed=0, backend="numpy-real")
    out["c1_tfim_n10_chi32"] = {"E": float(E), "energies": [float(e) for e in info["energies"]],
                               "free_fermion": float(tfim_free_fermion_energy(10, 1.0)),
                               "matvec_calls": int(info["matvec_calls"]),
                               "discarded_weight": float(info["discarded_weight"]),
                               "entropies": [float(s) for s in mps.entropies()],
                               "wall_s": time.perf_counter() - t0}
    be = get_backend("numpy-real")
    for N, chi, sweeps in ((12, 16, 4), (12, 64, 4), (64, 64, 3), (64, 128, 3)):
        W = open_chain(xxz_bulk(1.0), N)
        Wb, _ = to_block_mpo(W, [[1, -1]] * N, be, sym=U1())
        t0 = time.perf_counter()
        E, mps, info = dmrg(Wb, chi, charge=0, seed=1, n_sweeps=sweeps, tol=0, rtol=0,
                            expand=0, backend="numpy-real")
        ent, _ = _block_spectra(mps, [[1, -1]] * N)
        out[f"xxz_n{N}_chi{chi}"] = {
            "E": float(E), "energies": [float(e) for e in info["energies"]],
            "matvec_calls": int(info["matvec_calls"]), "sweep_s": info["sweep_s"],
            "discarded_weight": float(info["discarded_weight"]),
            "entropies": ent,
            "bonds": [{"charges": [int(c) for c in m.legs[2].charges],
                       "dims": [int(d) for d in m.legs[2].dims]} for m in mps],
            "wall_s": time.perf_counter() - t0}
        print(N, chi, E, flush=True)
    with open(os.path.join(HERE, "dmrg_small.json"), "w") as f:
        json.dump(out, f, indent=1)


def mode_c2(ref):
    from tnkit import dmrg, get_backend, U1, to_block_mpo
    N, chi = 64, 1024
    be = get_backend("numpy-real")
    W = open_chain(xxz_bulk(1.0), N)
    Wb, _ = to_block_mpo(W, [[1, -1]] * N, be, sym=U1())
    t0 = time.perf_counter()
    E, mps, info = dmrg(Wb, chi, charge=0, seed=1, n_sweeps=6, tol=0, rtol=0, expand=0,
                        backend="numpy-real", verbose=True)
    wall = time.perf_counter() - t0
    ent, spectra = _block_spectra(mps, [[1, -1]] * N)
    rec = {"E": float(E), "energies": [float(e) for e in info["energies"]],
           "matvec_calls": int(info["matvec_calls"]), "sweep_s": info["sweep_s"],
           "phase_time": info["phase_time"],
           "discarded_weight": float(info["discarded_weight"]),
           "entropies": ent,
           "mid_bond_spectrum": [float(x) for x in spectra[N // 2 - 1]],
           "bonds": [{"charges": [int(c) for c in m.legs[2].charges],
                      "dims": [int(d) for d in m.legs[2].dims]} for m in mps],
           "host": {"cpu_count": os.cpu_count(),
                    "omp": os.environ.get("OMP_NUM_THREADS")},
           "wall_s": wall}
    with open(os.path.join(HERE, "c2_xxz_n64_chi1024.json"), "w") as f:
        json.dump(rec, f, indent=1)
    print("E", E)


def mode_hubbard(ref):
    """U(1) x U(1) Hubbard runs of the reference (ProductSymmetry of two U(1)s)."""
    from tnkit import dmrg, get_backend, U1, to_block_mpo
    from tnkit.symmetry import ProductSymmetry
    from tnkit.block_backend import random_block_mps
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from tnkit_gb300.workloads import hubbard_mpo, HUBBARD_SITE_CHARGES
    sym = ProductSymmetry((U1(), U1()))
    be = get_backend("numpy-real")
    arrays, meta = {}, {}
    W = hubbard_mpo(6, 1.0, 4.0)
    Wb, _ = to_block_mpo(W, [list(HUBBARD_SITE_CHARGES)] * 6, be, sym=sym)
    w = Wb[2]
    meta["mpo_site2"] = {"legs": [{"charges": [list(c) for c in l.charges],
                                   "dims": list(l.dims), "sign": l.sign} for l in w.legs]}
    arrays["mpo_site2"] = np.asarray(w.data, dtype=np.float64)
    M = random_block_mps(Wb, 16, be, (3, 3), np.random.default_rng(1))
    meta["mps_seed1_chi16"] = [{"legs": [{"charges": [list(c) for c in l.charges],
                                          "dims": list(l.dims), "sign": l.sign}
                                         for l in m.legs]} for m in M]
    for i in (0, 2):
        arrays[f"mps_seed1_chi16_site{i}"] = np.asarray(M[i].data, dtype=np.float64)
    # exact ground energy of N=6 at half filling from the dense MPO
    T = W[0][0]
    for Wn in W[1:]:
        T = np.einsum("wab,wxcd->xacbd", T, Wn)
        T = T.reshape(T.shape[0], T.shape[1] * T.shape[2], -1)
    H = T[0]
    q = np.array([[0, 0], [1, 0], [0, 1], [1, 1]])
    import itertools
    idx = [i for i, ss in enumerate(itertools.product(range(4), repeat=6))
           if tuple(q[list(ss)].sum(0)) == (3, 3)]
    meta["n6_exact_E"] = float(np.linalg.eigvalsh(H[np.ix_(idx, idx)])[0])
    runs = {}
    for N, chi, sweeps in ((6, 16, 4), (8, 32, 3)):
        Wn = hubbard_mpo(N, 1.0, 4.0)
        Wbn, _ = to_block_mpo(Wn, [list(HUBBARD_SITE_CHARGES)] * N, be, sym=sym)
        t0 = time.perf_counter()
        E, mps, info = dmrg(Wbn, chi, charge=(N // 2, N // 2), seed=1, n_sweeps=sweeps, tol=0,
                            rtol=0, expand=0, backend="numpy-real")
        ent, _ = _block_spectra(mps, [list(HUBBARD_SITE_CHARGES)] * N)
        runs[f"n{N}_chi{chi}"] = {
            "E": float(E), "energies": [float(e) for e in info["energies"]],
            "discarded_weight": float(info["discarded_weight"]),
            "entropies": ent,
            "bonds": [{"charges": [list(c) for c in m.legs[2].charges],
                       "dims": [int(d) for d in m.legs[2].dims]} for m in mps],
            "wall_s": time.perf_counter() - t0}
        print(N, chi, E, flush=True)
    meta["runs"] = runs
    np.savez(os.path.join(HERE, "hubbard_u1u1.npz"), **arrays)
    with open(os.path.join(HERE, "hubbard_u1u1.json"), "w") as f:
        json.dump(meta, f, indent=1)


def mode_grad(ref):
    """dE/dJ_i by the reference's own observables (tnkit/dmrg_excited.py:185-211)."""
    from tnkit import dmrg, get_backend, U1, to_block_mpo
    from tnkit.block_backend import BlockBackend
    from tnkit.dmrg_excited import mpo_expectation
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from tnkit_gb300.workloads import xxz_disordered_mpo
    N, chi, delta = 10, 32, 1.0
    J = np.random.default_rng(2).uniform(0.5, 1.5, N - 1)
    be = get_backend("numpy")
    q = [[1, -1]] * N

    def ground(Jv):
        Wb, _ = to_block_mpo(xxz_disordered_mpo(Jv, delta), q, be, sym=U1())
        return dmrg(Wb, chi, charge=0, seed=1, n_sweeps=8, tol=1e-14, rtol=0, expand=0,
                    eig_tol=1e-12, backend=BlockBackend(be))
    E, mps, info = ground(J)
    grads = []
    for i in range(N - 1):
        e = np.zeros(N - 1)
        e[i] = 1.0
        Hb, _ = to_block_mpo(xxz_disordered_mpo(e, delta), q, be, sym=U1())
        grads.append(complex(mpo_expectation(mps, Hb)).real)
    h = 1e-5
    fd = {}
    for i in (0, 4, 8):
        Jp, Jm = J.copy(), J.copy()
        Jp[i] += h
        Jm[i] -= h
        fd[str(i)] = (float(ground(Jp)[0]) - float(ground(Jm)[0])) / (2 * h)
    rec = {"N": N, "chi": chi, "delta": delta, "J": [float(x) for x in J], "E": float(E),
           "hf_grad": grads, "fd_h": h, "fd_grad": fd, "backend": "numpy (complex128)"}
    with open(os.path.join(HERE, "grad_xxz10.json"), "w") as f:
        json.dump(rec, f, indent=1)
    print("E", E, "grads", grads)


def _dense_vector(mps):
    """The state vector of a block MPS with every leg in sector order (its flat amplitudes)."""
    v = np.ones((1,), complex)
    for t in mps:
        d = t.to_dense()
        v = np.tensordot(v.reshape(-1, d.shape[0]), d, (1, 0)).reshape(-1, d.shape[-1])
    return v.reshape(-1)


def mode_tdvp(ref):
    from tnkit import get_backend, U1, to_block_mpo, tdvp2_evolve
    from tnkit.block_backend import BlockBackend, random_block_mps
    from tnkit.eigensolver import lanczos_expm
    from tnkit._dmrg import apply_two_site
    arrays, meta = {}, {}
    N, chi, dt, steps = 10, 32, 0.05, 4
    be = get_backend("numpy")
    bb = BlockBackend(be)
    W = open_chain(xxz_bulk(1.0), N)
    Wb, _ = to_block_mpo(W, [[1, -1]] * N, be, sym=U1())
    mps = random_block_mps(Wb, 8, be, 0, np.random.default_rng(5))
    mps = [m.canonical() for m in mps]
    for i, m in enumerate(mps):
        arrays[f"init_{i}"] = np.asarray(m.data)
        meta[f"init_{i}"] = {"legs": _legs_json(m.struct), "charge": int(m.struct.charge)}
    out, rec = tdvp2_evolve(list(mps), Wb, chi, dt, steps, backend=bb)
    arrays["final_vector"] = _dense_vector(out)
    arrays["init_vector"] = _dense_vector(mps)
    meta["params"] = {"N": N, "chi": chi, "dt": dt, "n_steps": steps, "seed": 5, "chi0": 8}
    meta["final_bonds"] = [{"charges": [int(c) for c in m.legs[2].charges],
                            "dims": [int(d) for d in m.legs[2].dims]} for m in out]
    # the Krylov exponential alone: exp(-i dt/2 H) on a fixed vector of a 300x300 Hermitian H
    rng = np.random.default_rng(4)
    n = 300
    Q = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    H = 0.5 * (Q + Q.conj().T)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    info = {}
    y = lanczos_expm(lambda x: H @ x, v, -0.5j * 0.1, be, m=30, info=info)
    arrays["expm_H"], arrays["expm_v"], arrays["expm_y"] = H, v, np.asarray(y)
    meta["expm"] = {"tau_imag": -0.05, "m": 30, "krylov_dim": int(info["krylov_dim"]),
                    "err_est": float(info["err_est"])}
    np.savez_compressed(os.path.join(HERE, "tdvp_xxz10.npz"), **arrays)
    with open(os.path.join(HERE, "tdvp_xxz10.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print("wrote tdvp_xxz10.{npz,json}; krylov dim", info["krylov_dim"])


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("mode", choices=["small", "dmrg", "c2", "tdvp", "hubbard", "grad"])
    ap.add_argument("--ref", default=os.environ.get("TNKIT_REF"),
                    help="path of the reference tnkit checkout (or set TNKIT_REF)")
    a = ap.parse_args()
    if not a.ref:
        ap.error("give the reference checkout with --ref or the TNKIT_REF environment variable")
    ref = _import_ref(a.ref)
    {"small": mode_small, "dmrg": mode_dmrg, "c2": mode_c2, "tdvp": mode_tdvp,
     "hubbard": mode_hubbard, "grad": mode_grad}[a.mode](ref)
