"""Golden vectors of the binned-cell deposit, computed by the REFERENCE's own ``Cells`` accumulator
(sgl_full.py:1282-1533), run unmodified with ``oracle/numba_standin`` standing in for Numba (its
kernels then run as plain Python, operation for operation).

Two seeded builds of synthetic objects (point sets shaped like the emitters' output: kappa over
both signs and the whole fine lattice and beyond, gamma below the clip and above the lattice, points
exactly on the last edges, NaNs, an empty object, beta = 0, shear tangential or not):
  * build "plain": 3 shells, nord 3, no xi_lin term -- every deposit's histograms and totals;
  * build "xi": the xi_lin term on the reference's k_perp quadrature (xi_kperp_grid of the default
    cosmology, mmax 2) with the positive closure's rate deposit, two lens-redshift nodes with a shear
    tail each, closed by xi_end into compressed row groups.
Writes tests/golden/cells_ref.npz (committed, small): the inputs, the sparse histograms, N, dropped,
lin and the xi groups (singular values and rows^T rows f for seeded f, which fix the rows up to
sign and rotation within the kept subspace).

A third, larger record (``shell`` stage, not committed) is one real lens shell of the reference's z_s
build as tests/golden/make_fixtures.py makes it (elliptical truncated hosts, filaments, the exact subhalo
sector, the xi_lin nodes): every deposit the reference's emitters make into the shell's Cells, recorded
on the way in, with that Cells' outputs; written to tests/golden/full/cells_shell_zs<z>_s<i>.npz.

Usage:  python tests/golden/make_cells_golden.py --reference PATH   (or SGL_REFERENCE=PATH)
        python tests/golden/make_cells_golden.py shell --zs 1 --shell 40 --reference PATH
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
from _reference import reference_root  # noqa: E402

REPO = Path(__file__).resolve().parents[2]
NF = 3                      # test vectors per xi group


def objects(rng, n_obj, shells, with_R, nmax):
    """Seeded point sets; returns a list of dicts (K, G, W, R, shell, beta, tang)."""
    radii = np.exp(rng.uniform(np.log(1e-3), np.log(60.0), 300))
    out = []
    for o in range(n_obj):
        n = 0 if o == 3 else int(rng.integers(1, nmax))
        s = rng.random(n)
        K = np.where(s < 0.7, np.exp(rng.uniform(np.log(1e-9), np.log(45.0), n)),
                     -np.exp(rng.uniform(np.log(1e-9), np.log(1e-2), n)))
        G = np.exp(rng.uniform(np.log(1e-12), np.log(50.0), n))
        W = np.exp(rng.uniform(np.log(1e-6), np.log(1e2), n))
        if n > 10:
            K[0], G[1] = 30.0, 30.0              # on the last fine (and coarse) edges
            K[2] = -30.0                          # on the first edge
            G[3] = 0.0                            # below the clip
            K[4] = 1e-7                           # on an inner edge
        if n > 20 and o % 5 == 1:
            K[5], G[6] = np.nan, np.nan
        R = radii[rng.integers(0, radii.size, n)] if with_R else None
        beta = 0.0 if o == 7 else float(rng.uniform(0.4, 3.0))
        out.append(dict(K=K, G=G, W=W, R=R, shell=int(rng.integers(0, shells)), beta=beta,
                        tang=bool(o % 3 != 2)))
    return out


def sparse(a):
    f = np.flatnonzero(a.ravel())
    return f.astype(np.int64), a.ravel()[f]


def run_build(F, tag, nshell, nord, objs, xi=None, nodes=None, out=None):
    cells = F.Cells(nshell, nord, xi=xi)
    if nodes is None:
        for ob in objs:
            cells.add(ob["K"], ob["G"], ob["W"], ob["shell"], ob["beta"])
    else:
        for node in nodes:
            cells.xi_begin(node["dchi"])
            for o in node["objects"]:
                ob = objs[o]
                cells.add(ob["K"], ob["G"], ob["W"], ob["shell"], ob["beta"], R=ob["R"], tang=ob["tang"])
            cells.xi_add_shear_tail(*node["tail"])
            cells.xi_end(node["shell"])
    for name in ("H0", "H0k", "H0g", "Hc"):
        i, v = sparse(getattr(cells, name))
        out[f"{tag}_{name}_i"], out[f"{tag}_{name}_v"] = i, v
    out[f"{tag}_N"] = np.float64(cells.N)
    out[f"{tag}_dropped"] = np.float64(cells.dropped)
    keys = sorted(cells.lin)
    out[f"{tag}_lin_keys"] = np.array(keys, float).reshape(-1, 2)
    out[f"{tag}_lin_vals"] = np.array([cells.lin[k] for k in keys], float)
    gs = cells.xi_groups
    if gs:
        out[f"{tag}_xg_shell"] = np.array([g["shell"] for g in gs], np.int64)
        out[f"{tag}_xg_m"] = np.array([g["m"] for g in gs], np.int64)
        out[f"{tag}_xg_nidx"] = np.array([g["idx"].size for g in gs], np.int64)
        out[f"{tag}_xg_nrow"] = np.array([g["rows"].shape[0] for g in gs], np.int64)
        out[f"{tag}_xg_idx"] = np.concatenate([g["idx"] for g in gs]).astype(np.int64)
        # the rows themselves are fixed only up to sign and rotation within the kept subspace: keep
        # their norms (the singular values) and, for NF seeded vectors f per group, rows^T rows f
        S, P = [], []
        for gi, g in enumerate(gs):
            f = np.random.default_rng(1000 + gi).standard_normal((g["idx"].size + 1, NF))
            S.append(np.linalg.norm(g["rows"], axis=1))
            P.append((g["rows"].T @ (g["rows"] @ f)).ravel())
        out[f"{tag}_xg_S"] = np.concatenate(S)
        out[f"{tag}_xg_P"] = np.concatenate(P)
        w = [g for g in gs if "W" in g]
        out[f"{tag}_xg_W"] = np.concatenate([g["W"] for g in w]) if w else np.zeros(0)
        out[f"{tag}_xg_v0"] = np.concatenate([g["v0"] for g in w]) if w else np.zeros(0)
    print(tag, "points", sum(o["K"].size for o in objs), "N", cells.N, "groups", len(gs), flush=True)
    return cells


def pack_objects(objs, tag, out):
    n = np.array([o["K"].size for o in objs])
    out[f"{tag}_off"] = np.concatenate([[0], np.cumsum(n)]).astype(np.int64)
    for k in ("K", "G", "W"):
        out[f"{tag}_{k}"] = np.concatenate([o[k] for o in objs])
    if objs[0]["R"] is not None:
        out[f"{tag}_R"] = np.concatenate([o["R"] for o in objs])
    out[f"{tag}_shell"] = np.array([o["shell"] for o in objs], np.int64)
    out[f"{tag}_beta"] = np.array([o["beta"] for o in objs], float)
    out[f"{tag}_tang"] = np.array([o["tang"] for o in objs], bool)


def record_shell(zs, shell):
    """Records shell `shell` of the reference's z_s build (the settings of make_fixtures.build)."""
    from sgl_analytic import pipeline as PL, sgl_full as F, subhalos          # noqa: E402
    log = []

    class Recording(F.Cells):
        def add(self, K, G, W, shell, beta, R=None, tang=True, xi_linear=False):
            log.append(("add", np.array(K, float).ravel(), np.array(G, float).ravel(), np.array(W, float).ravel(),
                        None if R is None else np.array(R, float).ravel(), int(shell), float(beta), bool(tang),
                        bool(xi_linear)))
            return super().add(K, G, W, shell, beta, R=R, tang=tang, xi_linear=xi_linear)

        def xi_begin(self, dchi):
            log.append(("begin", float(dchi)))
            return super().xi_begin(dchi)

        def xi_add_shear_tail(self, beta, Gam, Rm, n_area):
            log.append(("tail", float(beta), float(Gam), float(Rm), float(n_area)))
            return super().xi_add_shear_tail(beta, Gam, Rm, n_area)

        def xi_end(self, shell):
            log.append(("end", int(shell)))
            return super().xi_end(shell)

    cos = PL.make_cosmology(None)
    sub = subhalos.SubhaloModel(cos, zs, None, split=10.0, sector="exact", clump_edge="r200",
                                exact_kw=dict(method="moments"))
    xi = F.xi_kperp_grid(cos)
    ctx = F._make_ctx(cos, zs, [zs], 1, True, True, 12, 260, None, sub, 1e-8, "r200", "midpoint", 2, xi)
    F.Cells = Recording
    out = F._shell_pieces(ctx, shell)
    if any(e[0] == "add" and e[8] for e in log):
        raise SystemExit("the shell made xi_linear deposits, which the GPU deposit does not take")
    adds = [e for e in log if e[0] == "add"]
    rec = dict(zs=np.float64(zs), shell=np.int64(shell), nord=np.int64(1), xi_kp=xi["kp"], xi_c=xi["c"],
               xi_mmax=np.int64(xi["mmax"]))
    n = np.array([e[1].size for e in adds])
    rec["off"] = np.concatenate([[0], np.cumsum(n)]).astype(np.int64)
    for j, k in ((1, "K"), (2, "G"), (3, "W"), (4, "R")):
        rec[k] = np.concatenate([e[j] for e in adds])
    rec["obj_shell"] = np.array([e[5] for e in adds], np.int64)
    rec["obj_beta"] = np.array([e[6] for e in adds])
    rec["obj_tang"] = np.array([e[7] for e in adds], bool)
    # the event sequence: 0 begin (value dchi), 1 objects [a, b) (values a, b), 2 tail, 3 end
    ev, a = [], 0
    for e in log:
        if e[0] == "add":
            if ev and ev[-1][0] == 1:
                ev[-1][2] += 1
            else:
                ev.append([1, a, a + 1, 0.0, 0.0])
            a += 1
        elif e[0] == "begin":
            ev.append([0, e[1], 0, 0, 0])
        elif e[0] == "tail":
            ev.append([2, e[1], e[2], e[3], e[4]])
        else:
            ev.append([3, e[1], 0, 0, 0])
    rec["events"] = np.array(ev, float)
    pc = out[0]
    rec.update(ref_idx=pc["idx"], ref_h0=pc["h0"], ref_h0k=pc["h0k"], ref_h0g=pc["h0g"], ref_Hc=pc["Hc"],
               ref_N=np.float64(pc["N"]), ref_dropped=np.float64(pc["dropped"]))
    keys = sorted(pc["lin"])
    rec["ref_lin_beta"] = np.array(keys, float)
    rec["ref_lin_vals"] = np.array([pc["lin"][k] for k in keys])
    gs = pc["xi_groups"]
    rec["ref_xg_m"] = np.array([g["m"] for g in gs], np.int64)
    rec["ref_xg_nidx"] = np.array([g["idx"].size for g in gs], np.int64)
    rec["ref_xg_nrow"] = np.array([g["rows"].shape[0] for g in gs], np.int64)
    rec["ref_xg_idx"] = np.concatenate([g["idx"] for g in gs]).astype(np.int64) if gs else np.zeros(0, np.int64)
    rec["ref_xg_rows"] = np.concatenate([g["rows"].ravel() for g in gs]) if gs else np.zeros(0)
    path = REPO / "tests" / "golden" / "full" / f"cells_shell_zs{zs:g}_s{shell}.npz"
    path.parent.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(path, **rec)
    print("shell", shell, "objects", len(adds), "points", int(n.sum()), "groups", len(gs), "->", path, flush=True)


def main():
    ref = reference_root()
    if len(sys.argv) > 1 and sys.argv[1] == "shell":
        for p in (str(ref / "src"), str(REPO / "oracle" / "numba_standin")):
            sys.path.insert(0, p)
        args = sys.argv[2:]
        zs = float(args[args.index("--zs") + 1]) if "--zs" in args else 1.0
        shell = int(args[args.index("--shell") + 1]) if "--shell" in args else 40
        record_shell(zs, shell)
        return
    for p in (str(ref / "src"), str(REPO / "oracle" / "numba_standin")):
        sys.path.insert(0, p)
    from sgl_analytic import pipeline as PL, sgl_full as F          # noqa: E402
    out = {}
    rng = np.random.default_rng(20261204)
    objs = objects(rng, 30, 3, False, 2500)
    pack_objects(objs, "plain", out)
    run_build(F, "plain", 3, 3, objs, out=out)

    cos = PL.make_cosmology(None)
    xi = F.xi_kperp_grid(cos)
    xi["pos"] = True
    objs = objects(rng, 24, 2, True, 1000)
    pack_objects(objs, "xi", out)
    nodes = [dict(dchi=37.5, shell=0, objects=list(range(0, 12)), tail=(1.3, 2.0e-3, 4.0, 0.8)),
             dict(dchi=52.0, shell=1, objects=list(range(12, 24)), tail=(0.9, 5.0e-4, 9.0, 1.7))]
    out["xi_node_obj"] = np.array([n["objects"][0] for n in nodes] + [nodes[-1]["objects"][-1] + 1], np.int64)
    out["xi_node_dchi"] = np.array([n["dchi"] for n in nodes])
    out["xi_node_shell"] = np.array([n["shell"] for n in nodes], np.int64)
    out["xi_node_tail"] = np.array([n["tail"] for n in nodes])
    out["xi_kp"], out["xi_c"] = xi["kp"], xi["c"]
    out["xi_mmax"] = np.int64(xi["mmax"])
    run_build(F, "xi", 2, 3, objs, xi=xi, nodes=nodes, out=out)
    np.savez_compressed(REPO / "tests" / "golden" / "cells_ref.npz", **out)


if __name__ == "__main__":
    main()
