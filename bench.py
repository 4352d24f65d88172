#!/usr/bin/env python
"""Benchmark of the e-ph vertex path: |g|^2 vertices/s of RTA-rate requests.

Workload (the one the metric is quoted on): synthetic diamond-Si-like fcc
2-atom crystal, a = 5.43 A, 28 amu, nw = 8 Wannier bands, nb = 6 modes, Re and
Rp Wigner-Seitz sets of a 6x6x6 supercell (279 cells each), 24^3 k = q mesh,
window +-0.5 eV around mu = mid-gap + 0.6 eV, Gaussian delta sigma = 10 meV,
T = 300 K.  A step is one full RTA-rate request (H(k) and D(q) set-up and
eigensolves, g(Re,Rp) -> g(k,Rp), the Rp Fourier, rotations, |g|^2, delta x
occupations, compensated rate sums) in the split-FP32 (3xTF32) tcgen05 form.

Our arm: ``value`` is vertices/s with the Wannier data resident in HBM, from
the library's CUDA events on its launch stream; ``e2e`` is the same metric for
the one-shot drop-in through the C ABI from pinned host buffers (create ->
rates -> destroy, every host<->device copy inside the timed region).
``--impl reference``: the reference algorithm on the host cores (the CPU
restatement of the reference path, literal per-vertex g2, OpenMP over k').

One GPU per call: the library's fused kernels share operand tiles between
the two CTAs of a cluster by TMA multicast within this GPU's memory, and the
path runs on one image and one GPU.  Under torchrun with more than one rank
the GPU arm does no work and rank 0 prints a line saying so; the reference
arm (host cores only) runs on rank 0.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "|g|^2 vertices/s (split-FP32 3xTF32 tcgen05, RTA rates within 1e-6 of FP64)"
UNIT = "vertices/s"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thr = threading.Thread(target=self._read, daemon=True)
            self.thr.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clocks not sampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, n in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower() == "active":
                    reasons.add(n)
        loaded = [x for x in sm if mx and x > 0.3 * max(mx)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons), "samples": len(self.rows)}


MESH = (24, 24, 24)


def workload():
    from elphbolt_gb300 import synthetic as S
    wd = S.si_like()                                   # seed 20260101, 6^3 WS supercell
    req = S.si_like_request(wd, MESH)                  # 24^3, +-0.5 eV at mid-gap+0.6 eV, 10 meV
    return wd, req


def config_dict(wd, req):
    """The workload, identical in both arms (run statistics go to ``stats``)."""
    c = {"workload": "Si-like fcc 2-atom, nwann 8, nmodes 6, %d Re / %d Rp WS cells (6^3), 24^3 k=q mesh, "
                     "window +-0.5 eV at mid-gap+0.6 eV, Gaussian delta 10 meV, T 300 K" % (wd.nwsk, wd.nwsq),
         "mesh": list(req.mesh), "nwann": wd.numwannbands, "nmodes": wd.numbranches,
         "n_ws_re": wd.nwsk, "n_ws_rp": wd.nwsq, "precision": "split-FP32 (3xTF32, FP32 accumulate)",
         "l2_policy": "inputs larger than L2 (g(Re,Rp) TF32 planes 494 MB, stage-B operand planes 2.9 GB)"}
    return c


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("bf16_tflops"), d.get("hbm_gbs"), "measured"
    return 1900.0, 6800.0, "fallback"


def tf32_cublas_tflops(n=8192, reps=10):
    """Dense TF32 tensor throughput of this GPU, measured live: cuBLAS SGEMM with
    TF32 tensor ops (torch.matmul, allow_tf32), n^3, best of `reps` (CUDA events)."""
    import torch
    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    try:
        a = torch.randn(n, n, device="cuda", dtype=torch.float32)
        b = torch.randn(n, n, device="cuda", dtype=torch.float32)
        for _ in range(3):
            torch.matmul(a, b)
        best = None
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        del a, b
        return 2.0 * n ** 3 / (best * 1e-3) / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = old


def traffic_per_gflop():
    """DRAM bytes per algorithmic GFLOP of the fused stage-B kernel, from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "stageB_fused86_traffic.json")
    if os.path.exists(p):
        try:
            return json.load(open(p)).get("dram_bytes_per_alg_gflop")
        except Exception:
            return None
    return None


def cpu_sample(wd, req, seconds_target=20.0, states=None):
    """The CPU oracle (literal per-vertex g2) on a bounded sample of initial states."""
    from oracle import oracle as O
    ncores = os.cpu_count() or 1
    W = O.Wannier(wd)
    t0 = time.time()
    R = O.RatesRun(W, req, nthreads=ncores)
    t_setup = time.time() - t0
    # calibrate: one state, then enough states for ~seconds_target
    a = R.run(0, 1)
    per_state_s = a["us_loop"] * 1e-6
    n = states or max(1, min(64, int(seconds_target / max(per_state_s, 1e-3))))
    b = R.run(1, n)
    R.close()
    v = b["vertices"]
    t = b["us_loop"] * 1e-6
    # the oracle's rates of initial states 0 .. n (zero elsewhere), for the parity check
    return dict(value=v / t, cores=ncores, states=n, vertices=v, seconds=t, setup_s=t_setup,
                nstates_total=a["nstates_inwindow"], rates=a["rates"] + b["rates"], indexlist=b["indexlist"])


def error_vs_oracle(cpu, gpu_idx, forms):
    """Largest relative error per rate of each GPU form against the oracle, on
    the initial states the oracle ran (the CPU sample)."""
    import numpy as np
    if not np.array_equal(cpu["indexlist"], gpu_idx):
        return {"error": "window k lists differ"}
    ref = cpu["rates"]
    m = ref > 0
    out = {"states": int(m.sum()), "what": "GPU rates vs the CPU oracle (FP64, literal per-vertex g2) on the "
                                         "states of the cpu_baseline sample, full k' sums"}
    for name, r in forms.items():
        out[name + "_max_rel"] = float(np.max(np.abs(r[m] - ref[m]) / ref[m]))
    return out


def cpu_sample_ph(wd, req, seconds_target=10.0):
    """The CPU oracle's phonon side (ibzq loop: gReq per q, literal 'el' g2 per
    vertex) on a bounded sample of q-points."""
    from oracle import oracle as O
    ncores = os.cpu_count() or 1
    R = O.RatesRun(O.Wannier(wd), req, nthreads=ncores)
    a = R.run_ph(1, 1)                     # calibrate on one q (not Gamma)
    per_q_s = max(a["us_loop"] * 1e-6, 1e-3)
    n = max(1, min(64, int(seconds_target / per_q_s)))
    b = R.run_ph(2, n)
    R.close()
    t = b["us_loop"] * 1e-6
    return dict(value=b["vertices"] / t, cores=ncores, qpoints=n, vertices=b["vertices"], seconds=t)


def phonon_side(W, req, steps, el_ms, fp64_el_ms):
    """ephg_ph_rates on the bench request: both sides in one sweep (split), its
    cost over the electron side alone, and its phonon rates against the FP64 form."""
    import numpy as np
    from elphbolt_gb300 import _lib
    ms = []
    for _ in range(max(3, steps)):
        s = W.ph_rates(req, precision=_lib.PREC_SPLIT_TF32, electrons=True)
        ms.append(s["stats"]["ms_total"])
    f = W.ph_rates(req, precision=_lib.PREC_FP64, electrons=True)
    v = s["stats"]["vertices"]
    t = float(np.median(ms))
    ref = f["rates_phe"]
    m = ref > 0
    err = float(np.max(np.abs(s["rates_phe"][m] - ref[m]) / ref[m])) if m.any() else None
    return {"value": v / (t * 1e-3), "unit": UNIT, "ms_per_step": t,
            "el_only_ms_per_step": el_ms, "added_ms": t - el_ms,
            "fp64_ms_per_step": f["stats"]["ms_total"], "fp64_el_only_ms_per_step": fp64_el_ms,
            "split_speedup_vs_fp64": f["stats"]["ms_total"] / t,
            "rates_phe_max_rel_vs_fp64": err, "rates_phe_positive": int(m.sum()), "rates_phe_size": int(ref.size),
            "what": "ephg_ph_rates: ibzq 'g' + 'Y' + ph-e RTA rates (every q of the mesh x nb) and the electron "
                    "rates of the same vertices in one sweep; value = vertices/s of that sweep"}


def polar_side(steps):
    """The polar long-range terms (dyn_nonanalytic, long_range_prefac) on a
    SiC-like crystal (3C-SiC's lattice, masses, dielectric constant and Born
    charges; nw 8, 6^3 WS sets) with the bench request's mesh and window: both
    sides in one split sweep, its cost over the same crystal without the
    long-range terms, and its rates against the FP64 form."""
    import numpy as np
    from elphbolt_gb300 import _lib, synthetic as S
    from elphbolt_gb300.wannier import Wannier
    wd = S.make_wannier(S.make_crystal_sic_like(), 8, supercell=(6, 6, 6), seed=20260105)
    req = S.si_like_request(wd, MESH)
    W = Wannier(wd)
    try:
        split = lambda: W.ph_rates(req, precision=_lib.PREC_SPLIT_TF32, electrons=True)
        split()
        runs = [split() for _ in range(max(3, steps))]
        t = float(np.median([r["stats"]["ms_total"] for r in runs]))
        s = runs[-1]
        W.set_polar(None, None)
        W.el_rates(req, precision=_lib.PREC_SPLIT_TF32)
        t0 = float(np.median([W.el_rates(req, precision=_lib.PREC_SPLIT_TF32)["stats"]["ms_total"]
                              for _ in range(max(3, steps))]))
        W.set_polar(wd.crystal.epsilon, wd.crystal.born)
        f = W.ph_rates(req, precision=_lib.PREC_FP64, electrons=True)
    finally:
        W.deallocate_wannier()
    v = s["stats"]["vertices"]
    m, mp = f["rates"] > 0, f["rates_phe"] > 0
    rel_el = np.abs(s["rates"][m] - f["rates"][m]) / f["rates"][m]
    rel_ph = np.abs(s["rates_phe"][mp] - f["rates_phe"][mp]) / f["rates_phe"][mp]
    return {"workload": "SiC-like polar crystal (epsilon 7.419, Z* +-2.7515, nw 8, 6^3 WS), %dx%dx%d mesh" % MESH,
            "value": v / (t * 1e-3), "unit": UNIT, "vertices": v, "ms_per_step": t,
            "nonpolar_el_ms_per_step": t0, "setup_ms": s["stats"]["ms_setup"],
            "fp64_ms_per_step": f["stats"]["ms_total"], "split_speedup_vs_fp64": f["stats"]["ms_total"] / t,
            "rates_max_rel_vs_fp64": float(rel_el.max()), "rates_phe_max_rel_vs_fp64": float(rel_ph.max()),
            "rates_phe_p999_rel_vs_fp64": float(np.quantile(rel_ph, 0.999)),
            "what": "ephg_ph_rates with ephg_set_polar: both rate sets in one split sweep, long-range terms on"}


def symmetry_side(steps):
    """Crystal symmetry (ephg_set_symmetry): a symmetric model of the bench
    crystal -- Si-like fcc 2-atom cell, 4 s-like Wannier functions per atom
    (nw 8), central springs, bond-stretching e-ph coupling, 6^3 WS sets -- with
    the bench request's mesh and window.  The electron rates over the full
    zone and over the irreducible wedge (48 rotations), and the wedge's split
    rates against its FP64 form."""
    import numpy as np
    from elphbolt_gb300 import _lib, synthetic as S, symmetry as Y
    from elphbolt_gb300.wannier import Wannier
    wd = S.make_wannier_symmetric(S.make_crystal_si_like(), 4, supercell=(6, 6, 6), seed=20260106)
    req = S.si_like_request(wd, MESH)
    R, _ = Y.crystal_symmetry(wd.crystal)
    W = Wannier(wd)
    try:
        split = lambda: W.el_rates(req, precision=_lib.PREC_SPLIT_TF32)
        split()
        full = [split() for _ in range(max(3, steps))]
        W.set_symmetry(R)
        split()
        ibz = [split() for _ in range(max(3, steps))]
        f = W.el_rates(req, precision=_lib.PREC_FP64)
    finally:
        W.deallocate_wannier()
    tf = float(np.median([r["stats"]["ms_total"] for r in full]))
    ti = float(np.median([r["stats"]["ms_total"] for r in ibz]))
    s, st = ibz[-1], ibz[-1]["stats"]
    m = f["rates"] > 0
    err = float(np.max(np.abs(s["rates"][m] - f["rates"][m]) / f["rates"][m])) if m.any() else None
    return {"workload": "symmetric Si-like model (4 s orbitals per atom, nw 8, 6^3 WS), %dx%dx%d mesh" % MESH,
            "rotations": len(R), "full_zone_ms_per_step": tf, "ibz_ms_per_step": ti, "speedup": tf / ti,
            "full_zone_rows": full[-1]["nwv"], "ibz_rows": s["nwv"], "full_zone_vertices": full[-1]["stats"]["vertices"],
            "ibz_vertices": st["vertices"], "ibz_stage_ms": {"setup": st["ms_setup"], "stage_a": st["ms_stage_a"],
                                                             "stage_bc": st["ms_stage_bc"]},
            "fp64_ibz_ms_per_step": f["stats"]["ms_total"], "ibz_rates_max_rel_vs_fp64": err,
            "what": "ephg_set_symmetry + ephg_el_rates: initial states on the irreducible window points"}


def large_side():
    """The large single instance: a 6-atom fcc cell (masses U[12, 60] amu),
    nw 32, nb 18, 279 Re / 279 Rp Wigner-Seitz cells (g(Re,Rp) 23 GB complex128,
    resident), a 40^3 k = q mesh, window +-0.1 eV about mid-gap + 0.6 eV,
    Gaussian 10 meV, 300 K, split form.  One warm-up request (operand planes),
    one timed; the rates of a sample of initial states against the CPU oracle
    (FP64, restructured form, full k' sums)."""
    import numpy as np
    from elphbolt_gb300 import _lib, synthetic as S
    from elphbolt_gb300.wannier import Wannier
    from oracle import oracle as O
    t0 = time.time()
    wd = S.large_instance()
    req = S.si_like_request(wd, (40, 40, 40), window=0.1)
    t_gen = time.time() - t0
    t1 = time.time()
    W = Wannier(wd)
    t_create = time.time() - t1
    try:
        W.el_rates(req, precision=_lib.PREC_SPLIT_TF32)
        out = W.el_rates(req, precision=_lib.PREC_SPLIT_TF32)
    finally:
        W.deallocate_wannier()
    st = out["stats"]
    ncores = os.cpu_count() or 1
    t2 = time.time()
    R = O.RatesRun(O.Wannier(wd), req, nthreads=ncores)
    t_oset = time.time() - t2
    a = R.run(0, 6, literal=False)
    R.close()
    ref = a["rates"]
    m = ref > 0
    err = float(np.max(np.abs(out["rates"][m] - ref[m]) / ref[m])) if m.any() else None
    same = bool(np.array_equal(a["indexlist"], out["indexlist"]))
    return {"workload": "6-atom fcc, nw 32, nb 18, %d Re / %d Rp WS cells (6^3; g 23 GB c128), 40^3 k=q mesh, "
                        "window +-0.1 eV at mid-gap+0.6 eV, Gaussian 10 meV, 300 K" % (wd.nwsk, wd.nwsq),
            "value": st["vertices"] / (st["ms_total"] * 1e-3), "unit": UNIT, "ms_per_step": st["ms_total"],
            "vertices": st["vertices"], "window_k": st["nwv"], "initial_states": st["nstates"],
            "stage_ms": {"setup": st["ms_setup"], "stage_a": st["ms_stage_a"], "stage_bc": st["ms_stage_bc"]},
            "contraction_tflops": (st["stage_a_gflop"] + st["stage_b_gflop"]) / st["ms_total"],
            "rates_max_rel_vs_oracle": err, "oracle_states": int(m.sum()), "window_lists_equal": same,
            "oracle_setup_s": t_oset, "generation_s": t_gen, "create_s": t_create,
            "what": "ephg_el_rates, split form (generic nw / nb path); error vs the CPU oracle on the first "
                    "initial states (full k' sums)"}


def batched_side(steps):
    """The batched form (ephg_el_rates_batch): 64 requests on 8 random crystals
    (nw 8-24, nb 6-18, WS sets of 93-279 vectors; meshes 8^3-16^3, windows
    0.2-1.0 eV), split form, 8 requests at a time with grouped GEMM launches.
    Against: the same 64 requests one at a time (split), the same batch without
    grouping, and the FP64 drop-in one at a time on one request per crystal
    (the one of median vertex count), which also gives the split form's error."""
    import numpy as np
    from elphbolt_gb300 import _lib, synthetic as S
    from elphbolt_gb300.wannier import Wannier, el_rates_batch
    t0 = time.time()
    wds, reqs = S.batch_workload()
    t_gen = time.time() - t0
    Ws = [Wannier(wd) for wd in wds]
    crys, rq = [Ws[c] for c, _ in reqs], [r for _, r in reqs]
    try:
        el_rates_batch(crys, rq, nslots=8)   # warm-up: operand planes, workspaces
        runs = [el_rates_batch(crys, rq, nslots=8) for _ in range(max(3, min(steps, 5)))]
        ungrouped = [el_rates_batch(crys, rq, nslots=8, grouped=False) for _ in range(2)]
        t1 = time.time()
        alone = [W.el_rates(r, precision=_lib.PREC_SPLIT_TF32) for W, r in zip(crys, rq)]
        t_alone = time.time() - t1
        outs = runs[-1][0]
        pick = []
        for c in range(len(wds)):
            mine = sorted((o["vertices"], i) for i, (cc, _) in enumerate(reqs) if cc == c for o in [outs[i]])
            pick.append(mine[len(mine) // 2][1])
        fp64_s, fp64_v, errs = 0.0, 0, []
        for i in pick:
            t2 = time.time()
            f = crys[i].el_rates(rq[i], precision=_lib.PREC_FP64)
            fp64_s += time.time() - t2
            fp64_v += f["vertices"]
            m = f["rates"] > 0
            errs.append(float(np.max(np.abs(outs[i]["rates"][m] - f["rates"][m]) / f["rates"][m])))
    finally:
        for W in Ws:
            W.deallocate_wannier()
    bs = [r[1] for r in runs]
    wall = float(np.median([b["wall_ms"] for b in bs]))
    verts = bs[-1]["vertices"]
    same = all(np.array_equal(a["rates"], o["rates"]) for a, o in zip(alone, outs))
    gv = verts / (wall * 1e-3)
    # algorithmic contraction work of the batch (stages A + B, complex MACs x 8)
    gflop = float(sum(o["stats"]["stage_a_gflop"] + o["stats"]["stage_b_gflop"] for o in outs))
    return {"workload": "64 requests on 8 random crystals (nw 8/16/24, nb 6/12/18, WS 93-279), meshes 8^3-16^3, "
                        "windows 0.2-1.0 eV, Gaussian 10 meV, 300 K",
            "crystals": [[wd.numwannbands, wd.numbranches, int(wd.rcells_k.shape[0])] for wd in wds],
            "vertices_per_batch": verts, "ms_per_batch": wall, "value": gv, "unit": UNIT,
            "contraction_gflop_per_batch": gflop, "contraction_tflops_over_wall": gflop / wall,
            "group": {k: bs[-1][k] for k in ("group_launches", "group_problems", "group_tiles", "max_group")},
            "ungrouped_ms_per_batch": float(np.median([b[1]["wall_ms"] for b in ungrouped])),
            "one_at_a_time_split_ms": t_alone * 1e3,
            "one_at_a_time_split_value": verts / t_alone,
            "fp64_dropin_one_at_a_time": {"value": fp64_v / fp64_s, "unit": UNIT, "requests": len(pick),
                                          "vertices": fp64_v, "seconds": fp64_s},
            "speedup_vs_fp64_dropin": gv / (fp64_v / fp64_s),
            "rates_max_rel_vs_fp64": max(errs), "results_equal_alone": same,
            "peak_workspace_bytes": bs[-1]["peak_workspace_bytes"], "generation_s": t_gen,
            "what": "ephg_el_rates_batch, 8 slots, grouped tcgen05 GEMM launches; host wall time per batch"}


def run_reference(args, ws, rank):
    if rank != 0:
        return 0
    wd, req = workload()
    from oracle import oracle as O
    O.build()
    ncores = os.cpu_count() or 1
    W = O.Wannier(wd)
    t0 = time.time()
    R = O.RatesRun(W, req, nthreads=ncores)
    t_setup = time.time() - t0
    a = R.run(0, 1)
    per_state_s = max(a["us_loop"] * 1e-6, 1e-3)
    budget = 150.0 / max(1, args.steps + args.warmup)       # whole run within a few minutes
    n = max(1, int(budget / per_state_s))
    s0 = 1
    for _ in range(args.warmup):
        R.run(s0, n)
        s0 += n
    tt, vv = 0.0, 0
    for _ in range(args.steps):
        b = R.run(s0, n)
        s0 += n
        tt += b["us_loop"] * 1e-6
        vv += b["vertices"]
    R.close()
    val = vv / tt
    line = {"metric": METRIC, "value": val, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tt / max(1, args.steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": config_dict(wd, req),
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": ncores, "kind": "port",
                             "sample": "%d steps x %d initial states of %d (literal per-vertex g2, OpenMP over k'); "
                                       "set-up %.1f s excluded" % (args.steps, n, a["nstates_inwindow"], t_setup)},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args, ws, rank, local):
    import numpy as np
    import torch
    from elphbolt_gb300 import _lib, build
    build.build()
    from elphbolt_gb300.wannier import Wannier
    import ctypes as ct

    dev = 0
    torch.cuda.set_device(dev)
    wd, req = workload()
    W = Wannier(wd)
    prec = _lib.PREC_SPLIT_TF32
    for _ in range(args.warmup):
        out = W.el_rates(req, precision=prec)
    # ---- timed region: value (one rank: the barrier is the synchronize) ----
    torch.cuda.synchronize()
    dev_ms, launches, gemm_ms, gemm_n, wall0 = [], 0, 0.0, 0, time.time()
    with ClockSampler(int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or 0)) as clk:
        for _ in range(args.steps):
            out = W.el_rates(req, precision=prec)
            st = out["stats"]
            dev_ms.append(st["ms_total"])
            launches += st["kernel_launches"]
            gemm_ms += st["ms_gemm_b"]
            gemm_n += st["gemm_b_launches"]
        torch.cuda.synchronize()
        wall = time.time() - wall0
    st = out["stats"]
    vertices = st["vertices"]
    total_ms = float(sum(dev_ms))
    value = args.steps * vertices / (total_ms * 1e-3)
    split_rates = out["rates"]
    # ---- e2e: one-shot drop-in through the C ABI from pinned host buffers, same step count ----
    e2e = e2e_measure(wd, req, prec, args.steps, args.warmup)
    # ---- FP64 plain drop-in on the same request (one step) ----
    f = W.el_rates(req, precision=_lib.PREC_FP64)
    fst = f["stats"]
    fp64_value = fst["vertices"] / (fst["ms_total"] * 1e-3)
    ref = f["rates"]
    mask = ref > 0
    rate_err = float(np.max(np.abs(split_rates[mask] - ref[mask]) / ref[mask])) if mask.any() else None
    ph = phonon_side(W, req, args.steps, float(np.median(dev_ms)), fst["ms_total"])
    W.deallocate_wannier()
    # ---- roofline of the dominant kernel (stage-B 3xTF32 contraction fused with the rate epilogue) ----
    bf16, hbm, src = peaks()
    achieved = st["stage_b_gflop"] / (st["ms_gemm_b"] * 1e-3) / 1e3          # TFLOP/s algorithmic
    peak = bf16 / 2.0 / 3.0       # TF32 = 1/2 of BF16 dense; three TF32 products per FP32-accurate one
    try:
        tf32 = tf32_cublas_tflops()
    except Exception:
        tf32 = None
    clk = clk.summary()
    tpg = traffic_per_gflop()
    cpu = cpu_sample(wd, req)
    parity = error_vs_oracle(cpu, out["indexlist"], {"split": split_rates, "fp64": ref})
    cpu_ph = cpu_sample_ph(wd, req)
    ph["cpu_baseline"] = {"value": cpu_ph["value"], "unit": UNIT, "cores": cpu_ph["cores"], "kind": "port",
                          "sample": "%d q-points x %d branches, %d vertices in %.1f s (gReq per q, literal 'el' "
                                    "g2 per vertex, OpenMP over k within each q)" % (cpu_ph["qpoints"], wd.numbranches,
                                                                       cpu_ph["vertices"], cpu_ph["seconds"])}
    serving = None
    if not args.no_serving:   # the metric's p99 latency: the serving loop under a Poisson stream
        try:
            from elphbolt_gb300 import serve_bench
            serving = serve_bench.measure(wds=serve_bench.make_crystals(base=wd))
        except Exception as e:   # the main line is still printed
            serving = {"error": repr(e)}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (3xTF32 contractions) + f64 (eigensolves, sums)",
            "data": "synthetic (seeded, reference units and layouts)",
            "config": config_dict(wd, req),
            "stats": {"window_k": st["nwv"], "initial_states": st["nstates"], "vertices_per_step": vertices},
            "e2e": e2e,
            "gpu_launches": launches,
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak,
                         "traffic": (tpg * st["stage_b_gflop"] / max(1, st["gemm_b_launches"])) if tpg else None,
                         "kernel": "k_stageB_fused86 (stage B Rp Fourier on tcgen05 + rate epilogue)",
                         "peak_source": "%s bf16 %.1f TFLOP/s / 2 (TF32) / 3 (split), of %s" % (src, bf16, src),
                         "launches_per_step": st["gemm_b_launches"],
                         "ms_per_launch": st["ms_gemm_b"] / max(1, st["gemm_b_launches"]),
                         "mcycles_per_launch": (st["ms_gemm_b"] / max(1, st["gemm_b_launches"]) * clk["sm_mhz"] * 1e-3
                                                if clk.get("sm_mhz") else None),
                         "tf32_cublas_tflops_measured": tf32,
                         "frac_of_measured_tf32_over_3": (achieved / (tf32 / 3.0)) if tf32 else None},
            "cpu_baseline": {"value": cpu["value"], "unit": UNIT, "cores": cpu["cores"], "kind": "port",
                             "sample": "%d initial states of %d, %d vertices in %.1f s (literal per-vertex g2, "
                                       "OpenMP over k'); set-up %.1f s excluded" % (
                                           cpu["states"], cpu["nstates_total"], cpu["vertices"], cpu["seconds"],
                                           cpu["setup_s"])},
            "fp64_dropin": {"value": fp64_value, "unit": UNIT, "ms_per_step": fst["ms_total"],
                            "split_speedup": value / fp64_value},
            "error_vs_fp64": {"rates_max_rel": rate_err},
            "error_vs_oracle": parity,
            "stage_ms": {"setup": st["ms_setup"], "stage_a": st["ms_stage_a"], "stage_bc": st["ms_stage_bc"],
                         "gemm_a": st["ms_gemm_a"], "gemm_b": st["ms_gemm_b"]},
            "wall_s": wall,
            "clocks": clk}
    line["phonon_side"] = ph
    if not args.no_polar:
        try:
            line["polar"] = polar_side(args.steps)
        except Exception as e:   # the main line is still printed
            line["polar"] = {"error": repr(e)}
    if not args.no_symmetry:
        try:
            line["symmetry"] = symmetry_side(args.steps)
        except Exception as e:   # the main line is still printed
            line["symmetry"] = {"error": repr(e)}
    if not args.no_batched:
        try:
            line["batched"] = batched_side(args.steps)
        except Exception as e:   # the main line is still printed
            line["batched"] = {"error": repr(e)}
    if not args.no_large:
        try:
            line["large"] = large_side()
        except Exception as e:   # the main line is still printed
            line["large"] = {"error": repr(e)}
    if serving is not None:
        line["serving"] = serving
    print(json.dumps(line), flush=True)
    return 0


def e2e_measure(wd, req, prec, steps, warmup=0):
    """create -> el_rates -> destroy through the C ABI, inputs in pinned host memory;
    `warmup` untimed steps first, as for the resident measurement."""
    import ctypes as ct
    import numpy as np
    import torch
    from elphbolt_gb300 import _lib
    L = _lib.load()
    c = wd.crystal

    def pin(a, dtype):
        t = torch.from_numpy(np.ascontiguousarray(np.asfortranarray(np.asarray(a, dtype=dtype)).ravel(order="F")))
        return t.pin_memory()

    arrs = {k: pin(v, d) for k, v, d in [
        ("lat", c.lattvecs, np.float64), ("bas", c.basis, np.float64), ("mas", c.masses, np.float64),
        ("rk", wd.rcells_k, np.int64), ("rq", wd.rcells_q, np.int64), ("rg", wd.rcells_g, np.int64),
        ("dk", wd.elwsdeg, np.int64), ("dq", wd.phwsdeg, np.int64), ("dg", wd.gwsdeg, np.int64),
        ("H", np.asfortranarray(wd.Hwann), np.complex128),
        ("D", np.asfortranarray(wd.Dphwann), np.complex128), ("G", np.asfortranarray(wd.gwann), np.complex128)]}
    d = _lib.WannierDesc()
    d.numwannbands, d.numbranches = wd.numwannbands, wd.numbranches
    d.nwsk, d.nwsq, d.nwsg, d.numatoms = wd.nwsk, wd.nwsq, wd.nwsg, c.numatoms
    for i in range(3):
        d.coarse_qmesh[i] = int(wd.coarse_qmesh[i])
    dp = lambda t: ct.cast(t.data_ptr(), _lib.c_dp)
    ip = lambda t: ct.cast(t.data_ptr(), _lib.c_i64p)
    d.lattvecs, d.basis, d.masses = dp(arrs["lat"]), dp(arrs["bas"]), dp(arrs["mas"])
    d.rcells_k, d.rcells_q, d.rcells_g = ip(arrs["rk"]), ip(arrs["rq"]), ip(arrs["rg"])
    d.elwsdeg, d.phwsdeg, d.gwsdeg = ip(arrs["dk"]), ip(arrs["dq"]), ip(arrs["dg"])
    d.Hwann, d.Dphwann, d.gwann = dp(arrs["H"]), dp(arrs["D"]), dp(arrs["G"])
    r = _lib.RateRequest()
    for i in range(3):
        r.mesh[i] = int(req.mesh[i])
    r.enref, r.fsthick, r.chempot, r.T = req.enref, req.fsthick, req.chempot, req.T
    r.delta_kind, r.sigma, r.precision = int(req.delta_kind), float(req.sigma), int(prec)
    N = int(np.prod(req.mesh))
    rates = torch.zeros(N * wd.numwannbands, dtype=torch.float64).pin_memory()
    idx = torch.zeros(N, dtype=torch.int64).pin_memory()
    stats = _lib.RateStats()
    h2d = sum(t.numel() * t.element_size() for t in arrs.values())
    d2h = rates.numel() * 8 + idx.numel() * 8
    def step():
        h = ct.c_void_p()
        _lib.check(L.ephg_create(ct.byref(d), ct.byref(h)))
        _lib.check(L.ephg_el_rates(h, ct.byref(r), dp(rates), ip(idx), ct.byref(stats), None, None, None, 0))
        _lib.check(L.ephg_destroy(h))
        return stats.vertices

    for _ in range(warmup):
        step()
    vert = 0
    torch.cuda.synchronize()
    t0 = time.time()
    for _ in range(steps):
        vert += step()
    torch.cuda.synchronize()
    t = time.time() - t0
    return {"value": vert / t, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "steps": steps, "warmup": warmup, "ms_per_step": 1e3 * t / steps,
            "flow": "ephg_create (upload from pinned host) + ephg_el_rates (host rates out) + ephg_destroy"}


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-loop (p50 / p99 latency) measurement")
    ap.add_argument("--no-polar", action="store_true", help="skip the polar-crystal measurement")
    ap.add_argument("--no-symmetry", action="store_true", help="skip the crystal-symmetry measurement")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-form measurement")
    ap.add_argument("--no-large", action="store_true", help="skip the large-instance (nw 32, nb 18, 40^3) measurement")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    if ws > 1 or args.gpus > 1:
        # one image, one GPU: no work on any rank, one line from rank 0
        if rank == 0:
            print(json.dumps({"metric": METRIC, "unit": UNIT, "n_gpus": max(ws, args.gpus), "value": None,
                              "unavailable": "one GPU per call: the path runs on one image and one GPU, and its "
                                             "fused kernels use TMA multicast within one GPU's memory"}), flush=True)
        return 0
    return run_ours(args, ws, rank, local)


if __name__ == "__main__":
    sys.exit(main())
