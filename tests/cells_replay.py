"""Replays the golden deposit builds of tests/golden/cells_ref.npz through any accumulator with the
reference ``Cells`` interface (add, xi_begin, xi_add_shear_tail, xi_end) and compares the result
with the reference's outputs stored beside the inputs."""
from __future__ import annotations

import numpy as np

from tests.conftest import GOLDEN

NF = 3


def load():
    return dict(np.load(GOLDEN / "cells_ref.npz"))


def xi_dict(d):
    return dict(kp=d["xi_kp"], c=d["xi_c"], mmax=int(d["xi_mmax"]), pos=True)


def objects(d, tag):
    off = d[f"{tag}_off"]
    for o in range(off.size - 1):
        s = slice(off[o], off[o + 1])
        yield dict(K=d[f"{tag}_K"][s], G=d[f"{tag}_G"][s], W=d[f"{tag}_W"][s],
                   R=d[f"{tag}_R"][s] if f"{tag}_R" in d else None,
                   shell=int(d[f"{tag}_shell"][o]), beta=float(d[f"{tag}_beta"][o]),
                   tang=bool(d[f"{tag}_tang"][o]))


def replay(cells, d, tag, batched=False):
    """Deposits the build's objects; batched=True hands each node's objects over in one call
    (cells.add_many), else one add per object, as the reference's emitters do."""
    objs = list(objects(d, tag))
    if tag == "plain":
        if batched:
            cells.add_many(objs)
        else:
            for ob in objs:
                cells.add(ob["K"], ob["G"], ob["W"], ob["shell"], ob["beta"])
        return cells
    nobj = d["xi_node_obj"]
    for n in range(nobj.size - 1):
        cells.xi_begin(float(d["xi_node_dchi"][n]))
        group = objs[nobj[n]:nobj[n + 1]]
        if batched:
            cells.add_many(group)
        else:
            for ob in group:
                cells.add(ob["K"], ob["G"], ob["W"], ob["shell"], ob["beta"], R=ob["R"], tang=ob["tang"])
        cells.xi_add_shear_tail(*[float(v) for v in d["xi_node_tail"][n]])
        cells.xi_end(int(d["xi_node_shell"][n]))
    return cells


def dense(d, tag, name, shape):
    a = np.zeros(int(np.prod(shape)))
    a[d[f"{tag}_{name}_i"]] = d[f"{tag}_{name}_v"]
    return a.reshape(shape)


def check_histograms(cells, d, tag, rtol):
    """rtol = 0: bit for bit.  Otherwise per bin, relative to the bin's sum of |terms| (w > 0, and
    kappa of one sign within a bin, so the sums themselves)."""
    for name in ("H0", "H0k", "H0g", "Hc"):
        got = np.asarray(getattr(cells, name))
        want = dense(d, tag, name, got.shape)
        if rtol == 0:
            assert np.array_equal(got, want), name
        else:
            assert np.array_equal(got != 0, want != 0), name
            np.testing.assert_allclose(got, want, rtol=rtol, atol=0, err_msg=name)
    N, dropped = float(d[f"{tag}_N"]), float(d[f"{tag}_dropped"])
    if rtol == 0:
        assert cells.N == N and cells.dropped == dropped
    else:
        assert abs(cells.N - N) <= rtol * N and abs(cells.dropped - dropped) <= rtol * N
    keys = [tuple(k) for k in d[f"{tag}_lin_keys"]]
    assert sorted((int(s), b) for s, b in cells.lin) == sorted((int(s), b) for s, b in keys)
    scale = N * 30.0
    for (s, b), v in zip(keys, d[f"{tag}_lin_vals"]):
        got = cells.lin[(int(s), b)]
        assert (got == v) if rtol == 0 else abs(got - v) <= rtol * scale, (s, b, got, v)


def check_groups(groups, d, tag, tol, rtol_w=0.0):
    """The compressed xi rows: shells, m and occupied bins exactly, the bins' rates within rtol_w (0:
    bit for bit); singular values and rows^T rows f for the stored test vectors within tol of the
    group's largest."""
    assert len(groups) == d[f"{tag}_xg_m"].size
    io = so = po = wo = vo = 0
    for gi, g in enumerate(groups):
        ni, nr = int(d[f"{tag}_xg_nidx"][gi]), int(d[f"{tag}_xg_nrow"][gi])
        assert int(g["m"]) == d[f"{tag}_xg_m"][gi] and int(g["shell"]) == d[f"{tag}_xg_shell"][gi]
        assert np.array_equal(np.asarray(g["idx"]), d[f"{tag}_xg_idx"][io:io + ni])
        rows = np.asarray(g["rows"])
        S_want = d[f"{tag}_xg_S"][so:so + nr]
        S = np.linalg.norm(rows, axis=1)
        assert rows.shape[1] == ni + 1
        # a mode right at the 1e-6 cut may fall either side of it
        assert abs(rows.shape[0] - nr) <= 1, (gi, rows.shape[0], nr)
        n = min(nr, rows.shape[0])
        np.testing.assert_allclose(S[:n], S_want[:n], rtol=0, atol=tol * S_want[0])
        f = np.random.default_rng(1000 + gi).standard_normal((ni + 1, NF))
        P = rows.T @ (rows @ f)
        P_want = d[f"{tag}_xg_P"][po:po + (ni + 1) * NF].reshape(ni + 1, NF)
        np.testing.assert_allclose(P, P_want, rtol=0, atol=tol * S_want[0] ** 2 * np.abs(f).max() * 4)
        if "W" in g:
            if rtol_w == 0:
                assert np.array_equal(np.asarray(g["W"]), d[f"{tag}_xg_W"][wo:wo + ni])
            else:
                np.testing.assert_allclose(np.asarray(g["W"]), d[f"{tag}_xg_W"][wo:wo + ni], rtol=rtol_w, atol=0)
            np.testing.assert_allclose(np.abs(g["v0"]), np.abs(d[f"{tag}_xg_v0"][vo:vo + d["xi_kp"].size]),
                                       rtol=0, atol=1e-9)
            wo += ni
            vo += d["xi_kp"].size
        io += ni
        so += nr
        po += (ni + 1) * NF


def shell_record():
    """The recorded real shell (tests/golden/make_cells_golden.py shell), or None when absent."""
    from tests.conftest import FULL_DIR
    paths = sorted(FULL_DIR.glob("cells_shell_zs1_s*.npz"))
    return dict(np.load(paths[0])) if paths else None


def replay_shell(cells, d):
    """The record's event sequence: node begin, runs of objects (one add_many each, or one add per
    object when the accumulator has no add_many), shear tails, node ends."""
    off = d["off"]
    for ev in d["events"]:
        kind = int(ev[0])
        if kind == 0:
            cells.xi_begin(ev[1])
        elif kind == 1:
            objs = []
            for o in range(int(ev[1]), int(ev[2])):
                s = slice(off[o], off[o + 1])
                objs.append(dict(K=d["K"][s], G=d["G"][s], W=d["W"][s], R=d["R"][s], shell=int(d["obj_shell"][o]),
                                 beta=float(d["obj_beta"][o]), tang=bool(d["obj_tang"][o])))
            if hasattr(cells, "add_many"):
                cells.add_many(objs)
            else:
                for ob in objs:
                    cells.add(ob["K"], ob["G"], ob["W"], ob["shell"], ob["beta"], R=ob["R"], tang=ob["tang"])
        elif kind == 2:
            cells.xi_add_shear_tail(*ev[1:5])
        else:
            cells.xi_end(int(ev[1]))
    return cells


def check_shell(c, d, rtol, tol_rows, exact=False):
    """The shell's lattices, totals and xi groups against the reference's outputs in the record."""
    h0, h0k, h0g = (np.asarray(getattr(c, n)).reshape(-1) for n in ("H0", "H0k", "H0g"))
    nz = np.flatnonzero((h0 != 0) | (h0k != 0) | (h0g != 0))
    assert np.array_equal(nz, d["ref_idx"])
    for name, h, ref in (("H0", h0, d["ref_h0"]), ("H0k", h0k, d["ref_h0k"]), ("H0g", h0g, d["ref_h0g"])):
        if exact:
            assert np.array_equal(h[d["ref_idx"]], ref), name
        else:
            np.testing.assert_allclose(h[d["ref_idx"]], ref, rtol=rtol, atol=1e-14 * np.abs(ref).max(), err_msg=name)
    Hc = np.asarray(c.Hc)[0]
    if exact:
        assert np.array_equal(Hc, d["ref_Hc"])
    else:
        np.testing.assert_allclose(Hc, d["ref_Hc"], rtol=rtol, atol=1e-14 * np.abs(d["ref_Hc"]).max())
    N = float(d["ref_N"])
    assert abs(c.N - N) <= 1e-12 * N
    assert abs(c.dropped - float(d["ref_dropped"])) <= 1e-12 * N
    for b, v in zip(d["ref_lin_beta"], d["ref_lin_vals"]):
        got = c.lin[(0, float(b))]
        assert abs(got - v) <= 1e-10 * abs(v) + 1e-12 * N, (b, got, v)
    gs = c.xi_groups
    assert [int(g["m"]) for g in gs] == d["ref_xg_m"].tolist()
    io = ro = 0
    for gi, g in enumerate(gs):
        ni, nr = int(d["ref_xg_nidx"][gi]), int(d["ref_xg_nrow"][gi])
        assert np.array_equal(np.asarray(g["idx"]), d["ref_xg_idx"][io:io + ni])
        ref_rows = d["ref_xg_rows"][ro:ro + nr * (ni + 1)].reshape(nr, ni + 1)
        rows = np.asarray(g["rows"])
        s0 = np.linalg.norm(ref_rows, axis=1).max()
        assert abs(rows.shape[0] - nr) <= 1
        f = np.random.default_rng(gi).standard_normal((ni + 1, 4))
        np.testing.assert_allclose(rows.T @ (rows @ f), ref_rows.T @ (ref_rows @ f), rtol=0,
                                   atol=tol_rows * s0 ** 2 * np.abs(f).max() * 4)
        io += ni
        ro += nr * (ni + 1)
