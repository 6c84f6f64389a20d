"""Run one parity case (tests/cases.py) through the CUDA library, the
reference kernels or the CPU oracle; every runner returns numpy arrays:
disp16, disp32, conf and, for the C-API cases, the cost volume ("cost") and
the aggregated volume ("acc") plus the column range where the reference
defines the aggregated volume ("acc_cols").  Test infrastructure only.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _oracle
from .cases import pair_for, parent_for


def acc_cols(case: dict) -> tuple[int, int]:
    """Columns where the reference's final aggregated volume is defined.

    Single-scale L->R aggregation leaves cost_acc unwritten left of
    minX1 = max(minD + D, 0) (reference src/sgm_kernels.cu:539-550); the
    R->L pass then adds to whatever the buffer held.  With numPaths >= 2 the
    same holds right of maxX1 = w + min(minD, 0).
    """
    if case["kind"] != "ss":
        return 0, case["w"]
    w = case["w"]
    minx1 = max(case["minD"] + case["D"], 0)
    maxx1 = w + min(case["minD"], 0)
    return (min(minx1, w), w) if case["paths"] == 1 else (min(minx1, w), max(min(maxx1, w), min(minx1, w)))


def inputs(case: dict):
    if "pair" in case:   # explicit images (the full-size configuration cases)
        left, right = case["pair"]
        return left, right, (None, None)
    left, right, truth = pair_for(case)
    parent = parent_for(case, truth) if case["kind"] == "level" and case["refine"] else (None, None)
    return left, right, parent


# ---------------------------------------------------------------------------
def run_oracle(case: dict, lut=None) -> dict:
    left, right, (pd, pc) = inputs(case)
    if case["kind"] == "ss":
        out = _oracle.orc_single_scale(left, right, case, lut)
    elif case["kind"] == "level":
        out = _oracle.orc_level(left, right, pd, pc, case, lut)
    else:
        out = _oracle.orc_matcher(left, right, lut, **case["params"])
    out["acc_cols"] = acc_cols(case)
    return out


def _torch():
    import torch
    return torch


def _dev(a):
    torch = _torch()
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def device_lut(case: dict) -> np.ndarray | None:
    """Adaptive-P2 table computed on the device (pyrsgm_gb300_p2_table)."""
    torch = _torch()
    from pyrsgm_gb300._native import lib
    if case["kind"] == "matcher":
        p = case["params"]
        if not p.get("adaptive_p2"):
            return None
        P2 = p.get("p2", 2400)
        a = (p.get("p2_alpha", 3.041), p.get("p2_beta", 16.137), p.get("p2_lower_mult", 0.601),
             p.get("p2_upper_mult", 1.77))
    else:
        if not case["adaptive"]:
            return None
        P2, a = case["P2"], case["p2p"]
    t = torch.zeros(256, dtype=torch.int32, device="cuda")
    assert lib().pyrsgm_gb300_p2_table(t.data_ptr(), P2, *a, torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    return t.cpu().numpy()


def run_mine(case: dict, with_volumes: bool = True) -> dict:
    torch = _torch()
    import pyrsgm_gb300 as pg
    left, right, (pd, pc) = inputs(case)
    h, w = left.shape
    L, R = _dev(left), _dev(right)
    d16 = torch.zeros((h, w), dtype=torch.int16, device="cuda")
    d32 = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    cf = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    out = {}
    if case["kind"] == "matcher":
        m = pg.StereoMatcher(w, h, pg.Params(**case["params"]))
        m.compute_into(L, R, d16, d32, cf)
        torch.cuda.synchronize()
        m.close()
    else:
        ws = pg.Workspace()
        if with_volumes:
            ws.set_debug(1)
        a = case["p2p"]
        if case["kind"] == "ss":
            r = pg.compute_single_scale(ws, L, R, d16, d32, cf, num_disparities=case["D"], min_disparity=case["minD"],
                                        block_size=case["bs"], p1=case["P1"], p2=case["P2"], uniqueness=case["uniq"],
                                        disp12_max_diff=case["maxdiff"], pre_filter_cap=case["pfc"],
                                        cost_mode=case["cost"], post_flags=case["post"], num_paths=case["paths"],
                                        adaptive_p2=case["adaptive"], p2_alpha=a[0], p2_beta=a[1], p2_lower=a[2],
                                        p2_upper=a[3])
        else:
            PD = _dev(pd) if pd is not None else None
            PC = _dev(pc) if pc is not None else None
            r = pg.compute_level(ws, L, R, PD, PC, d16, d32, cf, num_disparities=case["D"], min_disparity=0,
                                 max_disparity=case["maxD"], block_size=case["bs"], p1=case["P1"], p2=case["P2"],
                                 uniqueness=case["uniq"], disp12_max_diff=case["maxdiff"],
                                 pre_filter_cap=case["pfc"], cost_mode=case["cost"], post_flags=case["post"],
                                 num_paths=case["paths"], refine=case["refine"], min_confidence=case["minConf"],
                                 adaptive_p2=case["adaptive"], p2_alpha=a[0], p2_beta=a[1], p2_lower=a[2],
                                 p2_upper=a[3])
        assert r == 0
        if with_volumes:
            cost, acc = ws.volumes()
            torch.cuda.synchronize()
            out["cost"], out["acc"] = cost.cpu().numpy(), acc.cpu().numpy()
        torch.cuda.synchronize()
        ws.close()
    out.update(disp16=d16.cpu().numpy(), disp32=d32.cpu().numpy(), conf=cf.cpu().numpy(), acc_cols=acc_cols(case))
    return out


def _ref_matcher(case, L, R, d16, d32, cf):
    """StereoMatcher::compute schedule (reference src/stereo_matcher.cpp:238-338)
    driving the reference kernels; geometry from the oracle's restatement."""
    torch = _torch()
    ref = _oracle.ref()
    p = dict(case["params"])
    v = _oracle.orc_validate(**p)
    info = _oracle.orc_geometry(case["w"], case["h"], **p)
    levels = v["pyramid_levels"]
    st = torch.cuda.current_stream().cuda_stream
    args = (v["p2_alpha"], v["p2_beta"], v["p2_lower_mult"], v["p2_upper_mult"])

    def post(level):
        if level != 0:
            return 1
        return (1 if v["lr_check"] else 0) | (2 if v["median_filter"] else 0)

    wss = [ref.ref_create_workspace() for _ in range(levels + 1)]
    if levels == 0:
        h, w = case["h"], case["w"]
        r = ref.ref_compute_single_scale(wss[0], L.data_ptr(), R.data_ptr(), d16.data_ptr(), d32.data_ptr(),
                                         cf.data_ptr(), w, w, w * 2, w * 4, w * 4, w, h, v["num_disparities"],
                                         v["min_disparity"], v["block_size"], v["p1"], v["p2"],
                                         v["uniqueness_ratio"], v["disp12_max_diff"], v["pre_filter_cap"],
                                         v["cost_mode"], post(0), v["num_paths"], v["adaptive_p2"], *args, st)
        assert r == 0, ref.ref_last_error()
    else:
        pl, pr, pdisp, pconf = {}, {}, {}, {}
        pl[0], pr[0] = L, R
        for l in range(1, levels + 1):
            li = info[l]
            pl[l] = torch.empty((li["height"], li["width"]), dtype=torch.uint8, device="cuda")
            pr[l] = torch.empty_like(pl[l])
            pdisp[l] = torch.empty((li["height"], li["width"]), dtype=torch.int16, device="cuda")
            pconf[l] = torch.empty((li["height"], li["width"]), dtype=torch.float32, device="cuda")
            par = info[l - 1]
            for src, dst in ((pl[l - 1], pl[l]), (pr[l - 1], pr[l])):
                assert ref.ref_pyrdown_u8(src.data_ptr(), par["width"], par["width"], par["height"], dst.data_ptr(),
                                          li["width"], li["width"], li["height"], st) == 0
        for l in range(levels, -1, -1):
            li = info[l]
            w, h = li["width"], li["height"]
            refine = li["refine"]
            o16 = d16 if l == 0 else pdisp[l]
            o32 = d32 if l == 0 else None
            oc = cf if l == 0 else pconf[l]
            pw = info[l + 1]["width"] if refine else 0
            ph = info[l + 1]["height"] if refine else 0
            r = ref.ref_compute_level(wss[l], pl[l].data_ptr(), pr[l].data_ptr(),
                                      pdisp[l + 1].data_ptr() if refine else None,
                                      pconf[l + 1].data_ptr() if refine else None,
                                      o16.data_ptr(), o32.data_ptr() if o32 is not None else None, oc.data_ptr(),
                                      w, w, pw * 2, pw * 4, w * 2, w * 4, w * 4, w, h, pw, ph, li["num_labels"],
                                      v["min_disparity"], li["max_disparity"], li["block_size"], v["p1"], v["p2"],
                                      v["uniqueness_ratio"], v["disp12_max_diff"], v["pre_filter_cap"],
                                      v["cost_mode"], post(l), v["num_paths"], 1 if refine else 0,
                                      v["pyramid_min_confidence"], v["adaptive_p2"], *args, st)
            assert r == 0, ref.ref_last_error()
    torch.cuda.synchronize()
    for ws in wss:
        ref.ref_destroy_workspace(ws)


def run_ref(case: dict) -> dict:
    torch = _torch()
    ref = _oracle.ref()
    left, right, (pd, pc) = inputs(case)
    h, w = left.shape
    L, R = _dev(left), _dev(right)
    d16 = torch.zeros((h, w), dtype=torch.int16, device="cuda")
    d32 = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    cf = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    out = {}
    st = torch.cuda.current_stream().cuda_stream
    if case["kind"] == "matcher":
        _ref_matcher(case, L, R, d16, d32, cf)
    else:
        ws = ref.ref_create_workspace()
        a = case["p2p"]
        if case["kind"] == "ss":
            r = ref.ref_compute_single_scale(ws, L.data_ptr(), R.data_ptr(), d16.data_ptr(), d32.data_ptr(),
                                             cf.data_ptr(), w, w, w * 2, w * 4, w * 4, w, h, case["D"], case["minD"],
                                             case["bs"], case["P1"], case["P2"], case["uniq"], case["maxdiff"],
                                             case["pfc"], case["cost"], case["post"], case["paths"],
                                             int(case["adaptive"]), *a, st)
        else:
            PD = _dev(pd) if pd is not None else None
            PC = _dev(pc) if pc is not None else None
            ph, pw = pd.shape if pd is not None else (0, 0)
            r = ref.ref_compute_level(ws, L.data_ptr(), R.data_ptr(), PD.data_ptr() if PD is not None else None,
                                      PC.data_ptr() if PC is not None else None, d16.data_ptr(), d32.data_ptr(),
                                      cf.data_ptr(), w, w, pw * 2, pw * 4, w * 2, w * 4, w * 4, w, h, pw, ph,
                                      case["D"], 0, case["maxD"], case["bs"], case["P1"], case["P2"], case["uniq"],
                                      case["maxdiff"], case["pfc"], case["cost"], case["post"], case["paths"],
                                      int(case["refine"]), case["minConf"], int(case["adaptive"]), *a, st)
        assert r == 0, ref.ref_last_error()
        n = (h, w, case["D"])
        cost = torch.empty(n, dtype=torch.int16, device="cuda")
        acc = torch.empty(n, dtype=torch.int16, device="cuda")
        assert ref.ref_copy_volumes(ws, cost.data_ptr(), acc.data_ptr(), st) == 0
        torch.cuda.synchronize()
        out["cost"], out["acc"] = cost.cpu().numpy(), acc.cpu().numpy()
        ref.ref_destroy_workspace(ws)
    out.update(disp16=d16.cpu().numpy(), disp32=d32.cpu().numpy(), conf=cf.cpu().numpy(), acc_cols=acc_cols(case))
    return out


def matcher_levels(w: int, h: int, params: dict, left: np.ndarray, right: np.ndarray) -> list[dict]:
    """The StereoMatcher::compute schedule (reference src/stereo_matcher.cpp:238-338)
    run level by level through the C API, once on this library and once on the
    reference kernels, each feeding its own coarser output to the next level.
    Returns one record per level (coarsest first) with both sides' outputs and
    volumes (cost and aggregated, as run_mine / run_ref give them), the
    pyramid images of both, and the level geometry."""
    torch = _torch()
    import pyrsgm_gb300 as pg
    ref = _oracle.ref()
    v = _oracle.orc_validate(**params)
    info = _oracle.orc_geometry(w, h, **params)
    levels = v["pyramid_levels"]
    assert levels >= 1
    st = torch.cuda.current_stream().cuda_stream
    p2a = (v["p2_alpha"], v["p2_beta"], v["p2_lower_mult"], v["p2_upper_mult"])

    def post(level):
        if level != 0:
            return 1
        return (1 if v["lr_check"] else 0) | (2 if v["median_filter"] else 0)

    img = {"mine": {0: (_dev(left), _dev(right))}, "ref": {0: (_dev(left), _dev(right))}}
    for l in range(1, levels + 1):
        li, par = info[l], info[l - 1]
        for side in ("mine", "ref"):
            pair = []
            for src in img[side][l - 1]:
                dst = torch.zeros((li["height"], li["width"]), dtype=torch.uint8, device="cuda")
                if side == "mine":
                    pg.pyrdown(src, dst)
                else:
                    assert ref.ref_pyrdown_u8(src.data_ptr(), par["width"], par["width"], par["height"],
                                              dst.data_ptr(), li["width"], li["width"], li["height"], st) == 0
                pair.append(dst)
            img[side][l] = tuple(pair)
    outs = {"mine": {}, "ref": {}}
    records = []
    for l in range(levels, -1, -1):
        li = info[l]
        lw, lh, D = li["width"], li["height"], li["num_labels"]
        refine = bool(li["refine"])
        rec = {"level": l, "w": lw, "h": lh, "D": D, "refine": refine}
        for side in ("mine", "ref"):
            d16 = torch.zeros((lh, lw), dtype=torch.int16, device="cuda")
            d32 = torch.zeros((lh, lw), dtype=torch.float32, device="cuda") if l == 0 else None
            cf = torch.zeros((lh, lw), dtype=torch.float32, device="cuda")
            par = outs[side].get(l + 1)
            pw = info[l + 1]["width"] if refine else 0
            ph = info[l + 1]["height"] if refine else 0
            L, R = img[side][l]
            kw = dict(num_disparities=D, min_disparity=v["min_disparity"], max_disparity=li["max_disparity"],
                      block_size=li["block_size"], p1=v["p1"], p2=v["p2"], uniqueness=v["uniqueness_ratio"],
                      disp12_max_diff=v["disp12_max_diff"], pre_filter_cap=v["pre_filter_cap"],
                      cost_mode=v["cost_mode"], post_flags=post(l), num_paths=v["num_paths"], refine=refine,
                      min_confidence=v["pyramid_min_confidence"], adaptive_p2=bool(v["adaptive_p2"]),
                      p2_alpha=p2a[0], p2_beta=p2a[1], p2_lower=p2a[2], p2_upper=p2a[3])
            if side == "mine":
                ws = pg.Workspace()
                ws.set_debug(1)
                assert pg.compute_level(ws, L, R, par[0] if refine else None, par[1] if refine else None,
                                        d16, d32, cf, **kw) == 0
                cost, acc = ws.volumes()
                torch.cuda.synchronize()
                ws.close()
            else:
                ws = ref.ref_create_workspace()
                r = ref.ref_compute_level(ws, L.data_ptr(), R.data_ptr(),
                                          par[0].data_ptr() if refine else None,
                                          par[1].data_ptr() if refine else None,
                                          d16.data_ptr(), d32.data_ptr() if d32 is not None else None, cf.data_ptr(),
                                          lw, lw, pw * 2, pw * 4, lw * 2, lw * 4, lw * 4, lw, lh, pw, ph, D,
                                          v["min_disparity"], li["max_disparity"], li["block_size"], v["p1"],
                                          v["p2"], v["uniqueness_ratio"], v["disp12_max_diff"],
                                          v["pre_filter_cap"], v["cost_mode"], post(l), v["num_paths"],
                                          1 if refine else 0, v["pyramid_min_confidence"], v["adaptive_p2"], *p2a,
                                          st)
                assert r == 0, ref.ref_last_error()
                cost = torch.empty((lh, lw, D), dtype=torch.int16, device="cuda")
                acc = torch.empty_like(cost)
                assert ref.ref_copy_volumes(ws, cost.data_ptr(), acc.data_ptr(), st) == 0
                torch.cuda.synchronize()
                ref.ref_destroy_workspace(ws)
            outs[side][l] = (d16, cf)
            rec[side] = dict(disp16=d16.cpu().numpy(), disp32=d32.cpu().numpy() if d32 is not None else None,
                             conf=cf.cpu().numpy(), cost=cost.cpu().numpy(), acc=acc.cpu().numpy(),
                             acc_cols=(0, lw), left=L.cpu().numpy(), right=R.cpu().numpy())
        records.append(rec)
    return records


def run_ref_pyrdown(src: np.ndarray) -> np.ndarray:
    torch = _torch()
    h, w = src.shape
    S = _dev(src)
    dst = torch.zeros(((h + 1) // 2, (w + 1) // 2), dtype=torch.uint8, device="cuda")
    assert _oracle.ref().ref_pyrdown_u8(S.data_ptr(), w, w, h, dst.data_ptr(), dst.shape[1], dst.shape[1],
                                        dst.shape[0], torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    return dst.cpu().numpy()


def compare(a: dict, b: dict, volumes: bool = True) -> list[str]:
    """Differences between two runner outputs: exact for integer outputs,
    1e-6 absolute for the float outputs (disp32, conf)."""
    bad = []
    if not np.array_equal(a["disp16"], b["disp16"]):
        n = int((a["disp16"] != b["disp16"]).sum())
        bad.append(f"disp16 differs at {n} px")
    for k in ("disp32", "conf"):
        if a.get(k) is not None and b.get(k) is not None:
            d = float(np.max(np.abs(a[k].astype(np.float64) - b[k].astype(np.float64))))
            if d > 1e-6:
                bad.append(f"{k} max abs diff {d}")
    if volumes and "cost" in a and "cost" in b:
        if not np.array_equal(a["cost"], b["cost"]):
            bad.append(f"cost volume differs at {int((a['cost'] != b['cost']).sum())} voxels")
        x0, x1 = a["acc_cols"]
        if not np.array_equal(a["acc"][:, x0:x1], b["acc"][:, x0:x1]):
            bad.append(f"aggregated volume differs at {int((a['acc'][:, x0:x1] != b['acc'][:, x0:x1]).sum())} voxels")
    return bad
