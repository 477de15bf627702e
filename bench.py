"""Benchmark: batched Helmholtz apply of a 16-orbital batch (k=9, prec 1e-6, absolute), nodes/s.

One step = one level-synchronous batched apply of all 16 orbitals (each with its own
mu_i = sqrt(-2 eps_i) operator and uneven tree) in norm-tiered mixed precision, inputs
resident in device memory.  Beside it: the plain FP64 GPU apply of the same batch, the
relative L2 error of every mixed output against the FP64 output, the end-to-end rate
through the C ABI with host buffers (upload + apply + download), and the CPU oracle
(OpenMP FP64) on a bounded sample of the same workload.

Synthetic inputs stand in for an SCF state: phi_i = p_i(r - R_i) exp(-a_i |r - R_i|^2) with
p_i a random cubic (20 N(0,1) coefficients), a_i log-uniform in [0.3, 20], R_i uniform in
[-2, 2]^3, normalized; eps_i uniform in [-2, -0.1]; numpy default_rng(20261203).

`--impl reference` times the CPU oracle alone (the reference's own CPU path, MRCPP, is not
available to build) on the same metric.
"""
import argparse
import gc
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

SEED = 20261203
ORDER, PREC = 9, 1e-6
# DRAM bytes (read + write) per item of each tier kernel in the mixed step (k=9): ncu capture of every
# tier launch of two mixed steps of the first 8 orbitals of the batch with the caches left warm
# (--cache-control none), divided by those launches' items; summarised with its command in
# profiles/dram_traffic_tiers_k10.md and re-captured whenever a tier kernel changes
DRAM_PER_ITEM = {"fp32": 2.45e3, "tf32": 0.43e3, "df32": 4.55e3}
NORB = 16
METRIC = "Helmholtz-apply nodes/s: batched mixed vs plain FP64 GPU at 1e-6 rel. error"


def cubic_monomials():
    return [(a, b, c) for a in range(4) for b in range(4) for c in range(4) if a + b + c <= 3]


def orbital_terms(rng):
    mons = cubic_monomials()
    out = []
    for _ in range(NORB):
        alpha = float(np.exp(rng.uniform(np.log(0.3), np.log(20.0))))
        R = rng.uniform(-2.0, 2.0, 3)
        coefs = rng.standard_normal(len(mons))
        out.append([(float(c), alpha, tuple(R), m) for c, m in zip(coefs, mons)])
    eps = rng.uniform(-2.0, -0.1, NORB)
    return out, np.sqrt(-2.0 * eps)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self):
        self.samples, self.proc = [], None
        self.t0 = self.t1 = None  # the timed region (perf_counter seconds)

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                          "-lms", "50", "-i", "0"], stdout=subprocess.PIPE, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.samples.append((time.perf_counter(), parts))

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def mark(self, start):
        if start:
            self.t0 = time.perf_counter()
        else:
            self.t1 = time.perf_counter()

    def summary(self):
        inside = [p for t, p in self.samples
                  if (self.t0 is None or t >= self.t0) and (self.t1 is None or t <= self.t1)]
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(s[0]) for s in inside if s[0].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in inside for i in range(4) if s[3 + i].lower() == "active"})
        pw = [float(s[2]) for s in inside if s[2].replace(".", "").isdigit()]
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(inside[0][1]) if inside[0][1].replace(".", "").isdigit() else None,
                "sm_mhz_min": min(sm) if sm else None, "power_w_max": max(pw) if pw else None,
                "reasons": reasons, "samples": len(inside)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


# The CPU sample both arms time: the complete adaptive apply of these orbitals of the batch.
# `--impl reference` runs it once per step; the GPU arm's cpu_baseline runs it until --cpu-s
# seconds have passed, and compares the GPU outputs of these orbitals with the oracle's.
CPU_SAMPLE = (0, 1, 2)


def workload_config():
    """The `config` both arms print (identical, so the two lines describe the same workload)."""
    return {"workload": "helmholtz-batch16-k9-prec1e-6", "orbitals": NORB, "order": ORDER, "prec": PREC,
            "basis": "interpolating", "box": "[-32,32]^3", "abs_prec": True,
            "cpu_sample": "orbitals %d..%d of the batch, complete adaptive apply each, oracle FP64 OpenMP"
                          % (CPU_SAMPLE[0], CPU_SAMPLE[-1])}


def cpu_sample(terms, mus, budget_s, keep=False):
    """Oracle (OpenMP FP64) Helmholtz applies of the CPU_SAMPLE orbitals, the whole sample
    repeated until budget_s seconds of apply time have passed (at least once).  Projection and
    operator setup are outside the timed part.  keep: also return the oracle output trees of
    the first pass (orbital index -> (keys, coefs, is_leaf))."""
    from oracle import pyoracle as po
    po.build()
    threads = os.cpu_count() or 1
    po.set_threads(threads)
    mra = po.MRA(ORDER)
    jobs = []
    for i in CPU_SAMPLE:
        phi = po.project_gauss(PREC, po.Tree(mra), terms[i], abs_prec=True)
        phi.rescale(1.0 / phi.norm())
        jobs.append((i, phi, po.helmholtz(mra, float(mus[i]), PREC)))
    nodes, dt, reps, kept = 0, 0.0, 0, {}
    while reps == 0 or dt < budget_s:
        for i, phi, op in jobs:
            out = po.Tree(mra)
            t0 = time.perf_counter()
            st = po.apply(PREC, out, op, phi, max_iter=-1, abs_prec=True)
            dt += time.perf_counter() - t0
            nodes += st["out_nodes"]
            if keep and reps == 0:
                kept[i] = out.export()
        reps += 1
    res = {"value": nodes / dt, "unit": "nodes/s", "cores": threads, "kind": "port",
           "sample": "orbitals %d..%d of the batch, complete adaptive apply each, %d pass(es): %d output nodes "
                     "in %.1f s" % (CPU_SAMPLE[0], CPU_SAMPLE[-1], reps, nodes, dt)}
    return (res, kept) if keep else res


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    rng = np.random.default_rng(SEED)
    terms, mus = orbital_terms(rng)
    vals = []
    for _ in range(args.warmup):
        cpu_sample(terms, mus, 0.0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s = cpu_sample(terms, mus, 0.0)  # one pass of the sample per step
        vals.append(s["value"])
    wall = time.perf_counter() - t0
    v = float(np.mean(vals))
    print(json.dumps({"impl": "reference", "metric": METRIC, "value": v, "unit": "nodes/s", "n_gpus": args.gpus,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * wall / max(args.steps, 1),
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                      "data": "synthetic", "config": workload_config(),
                      "cpu_baseline": {"value": v, "unit": "nodes/s", "cores": s["cores"], "kind": "port",
                                       "sample": s["sample"]},
                      "e2e": {"value": v, "unit": "nodes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def poly_orbitals(rng, n, lo, hi):
    """n orbitals p(r - R) exp(-a |r - R|^2): random cubic p (20 N(0,1) coefficients), a
    log-uniform in [lo, hi], R uniform in [-2, 2]^3."""
    mons = cubic_monomials()
    out = []
    for _ in range(n):
        alpha = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        R = rng.uniform(-2.0, 2.0, 3)
        out.append([(float(c), alpha, tuple(R), m) for c, m in zip(rng.standard_normal(len(mons)), mons)])
    return out


def other_configs(mw, device, world, sync, steps):
    """The other workloads of the benchmark definition, each timed on the GPU (CUDA events around
    `steps` repetitions after one untimed) beside its error against FP64 and the oracle, and the
    oracle's own rate on the host cores (cpu_baseline: OpenMP FP64, the same inputs).

    poisson_k7:   plain FP64 Poisson apply of 4 normalized Gaussians (k=7, prec 1e-5, relative)
    helmholtz_prec1e-5 / _prec1e-7: the 16-orbital batch at those precisions, mixed vs FP64
    exchange_528: 32 orbitals, all 528 pair products rho_ij = phi_i phi_j (multiply at prec/10,
                  absolute, max-norm estimates) then the Poisson apply of each (prec*10, absolute,
                  steered by phi_i, phi_j; ExchangePotential.cpp:166-204), mixed precision."""
    import math
    import torch

    from oracle import pyoracle as po
    po.build()
    po.set_threads(os.cpu_count() or 1)
    out = {}

    def timed(fn, n):
        fn()
        sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(n):
            r = fn()
        e1.record()
        sync()
        return e0.elapsed_time(e1) / n, r

    def rel_vs_oracle(mra, t, otree):
        k2, c2, _ = otree.export()
        o = mw.FunctionTree(mra).upload(k2, c2)
        d = mw.FunctionTree(mra)
        mw.add(-1.0, d, [(1.0, t), (-1.0, o)])
        return d.norm() / max(o.norm(), 1e-300), bool(np.array_equal(t.download()[0], k2))

    def rel_err(mra, a, r):
        d = mw.FunctionTree(mra)
        mw.add(-1.0, d, [(1.0, a), (-1.0, r)])
        return d.norm() / max(r.norm(), 1e-300)

    # ---- Poisson, one density, plain FP64 ----
    prec, rng = 1e-5, np.random.default_rng(SEED)
    alphas = np.exp(rng.uniform(np.log(0.5), np.log(50.0), 4))
    centres = rng.uniform(-2, 2, (4, 3))
    terms = [((a / math.pi) ** 1.5, float(a), tuple(c), (0, 0, 0)) for a, c in zip(alphas, centres)]
    mra, omra = mw.MultiResolutionAnalysis(7, device=device), po.MRA(7)
    orho = po.project_gauss(prec, po.Tree(omra), terms)
    rho = mw.FunctionTree(mra).upload(*orho.export()[:2])
    P = mw.PoissonOperator(mra, prec)
    V = mw.FunctionTree(mra)

    def step1():
        V.clear()
        return mw.apply(prec, V, P, rho, precision="fp64")

    ms, st = timed(step1, steps)
    oV = po.Tree(omra)
    t0 = time.perf_counter()
    ost = po.apply(prec, oV, po.poisson(omra, prec), orho)
    cpu_s = time.perf_counter() - t0
    e_or, same = rel_vs_oracle(mra, V, oV)
    pts = np.random.default_rng(SEED + 1).uniform(-4, 4, (300, 3))
    exact = np.array([sum(math.erf(math.sqrt(a) * np.linalg.norm(p - r)) / np.linalg.norm(p - r)
                          for a, r in zip(alphas, centres)) for p in pts])
    out["poisson_k7"] = {
        "value": st["out_nodes"] * world / (ms / 1e3), "unit": "nodes/s", "ms_per_step": ms, "dtype": "f64",
        "input_nodes": rho.nnodes, "output_nodes": st["out_nodes"], "items": st["items"],
        "rel_l2_vs_oracle": e_or, "node_set_identical_to_oracle": same,
        "erf_max_abs_err_rel": float(np.abs(V.evalf(pts) - exact).max() / np.abs(exact).max()),
        "cpu_baseline": {"value": ost["out_nodes"] / cpu_s, "unit": "nodes/s", "cores": po.get_threads(),
                         "kind": "port", "sample": "the same apply, complete (%.2f s)" % cpu_s}}

    # ---- the 16-orbital Helmholtz batch at prec 1e-5 and 1e-7 ----
    for prec in (1e-5, 1e-7):
        rng = np.random.default_rng(SEED)
        terms, mus = orbital_terms(rng)
        mra, omra = mw.MultiResolutionAnalysis(ORDER, device=device), po.MRA(ORDER)
        ophis, phis = [], []
        for t in terms:
            f = po.project_gauss(prec, po.Tree(omra), t, abs_prec=True)
            f.rescale(1.0 / f.norm())
            ophis.append(f)
            phis.append(mw.FunctionTree(mra).upload(*f.export()[:2]))
        ops = mw.HelmholtzOperator.batch(mra, mus, prec)
        o64 = [mw.FunctionTree(mra) for _ in phis]
        omx = [mw.FunctionTree(mra) for _ in phis]

        def stepb(outs, mode):
            for o in outs:
                o.clear()
            return mw.apply_batch([prec] * NORB, outs, ops, phis, abs_prec=True, precision=mode)

        ms64, st64 = timed(lambda: stepb(o64, "fp64"), 1)
        msmx, stmx = timed(lambda: stepb(omx, "mixed"), steps)
        oout = po.Tree(omra)
        t0 = time.perf_counter()
        ost = po.apply(prec, oout, po.helmholtz(omra, float(mus[0]), prec), ophis[0], abs_prec=True)
        cpu_s = time.perf_counter() - t0
        e_mx, same_mx = rel_vs_oracle(mra, omx[0], oout)
        e_64, same_64 = rel_vs_oracle(mra, o64[0], oout)
        out["helmholtz_prec%g" % prec] = {
            "value": stmx["out_nodes"] * world / (msmx / 1e3), "unit": "nodes/s", "ms_per_step": msmx,
            "dtype": "f64+df32+f32+tf32", "fp64": {"value": st64["out_nodes"] * world / (ms64 / 1e3),
                                                  "ms_per_step": ms64},
            "speedup_mixed_vs_fp64": ms64 / msmx,
            "input_nodes_total": int(sum(p.nnodes for p in phis)), "output_nodes": stmx["out_nodes"],
            "items": {"fp64": stmx["items_fp64"], "df32": stmx["items_df"], "fp32": stmx["items_fp32"],
                      "tf32": stmx["items_tf32"]},
            "rel_l2_vs_fp64_per_orbital_max": max(rel_err(mra, a, r) for a, r in zip(omx, o64)),
            "rel_l2_vs_oracle_orbital0": {"mixed": e_mx, "fp64": e_64, "node_sets_identical": same_mx and same_64},
            "cpu_baseline": {"value": ost["out_nodes"] / cpu_s, "unit": "nodes/s", "cores": po.get_threads(),
                             "kind": "port", "sample": "orbital 0, complete adaptive apply (%.2f s)" % cpu_s}}

    # ---- exchange-like: 528 pair products, then their Poisson applies ----
    prec = 1e-5
    rng = np.random.default_rng(SEED)
    orbs = poly_orbitals(rng, 32, 0.5, 10.0)
    mra, omra = mw.MultiResolutionAnalysis(7, device=device), po.MRA(7)
    phis = []
    for t in orbs:
        f = mw.project(prec, mw.FunctionTree(mra), t, abs_prec=True)
        f.rescale(1.0 / f.norm())
        phis.append(f)
    pairs = [(i, j) for i in range(32) for j in range(i, 32)]
    P = mw.PoissonOperator(mra, prec)
    pt = [[phis[i], phis[j]] if i != j else [phis[i]] for i, j in pairs]
    rhos = [mw.FunctionTree(mra) for _ in pairs]
    vmx = [mw.FunctionTree(mra) for _ in pairs]
    parts = {}

    def step4():
        for t in rhos + vmx:
            t.clear()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record()
        sm = mw.multiply_batch(prec / 10, rhos, 1.0, [phis[i] for i, _ in pairs], [phis[j] for _, j in pairs],
                               abs_prec=True, use_max_norms=True)
        e[1].record()
        sa = mw.apply_batch(prec * 10, vmx, [P] * len(pairs), rhos, prec_trees=pt, abs_prec=True, precision="mixed")
        e[2].record()
        parts["e"] = e
        return sm, sa

    ms4, (sm, sa) = timed(step4, max(1, steps // 3))
    e = parts["e"]
    mul_ms, app_ms = e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])
    v64 = [mw.FunctionTree(mra) for _ in pairs]
    mw.apply_batch(prec * 10, v64, [P] * len(pairs), rhos, prec_trees=pt, abs_prec=True, precision="fp64")
    worst = 0.0
    for a, b in zip(vmx, v64):
        d = mw.FunctionTree(mra)
        mw.add(-1.0, d, [(1.0, a), (-1.0, b)])
        worst = max(worst, d.norm() / max(b.norm(), 1.0))
    # four pairs against the oracle (multiply and FP64 apply from the same input trees), timed
    sample = [pairs[k] for k in (0, 37, 300, 527)]
    oP = po.poisson(omra, prec)
    orac = {"rho": 0.0, "V": 0.0}
    same = True
    cpu_s, cpu_nodes = 0.0, 0
    for (i, j) in sample:
        k = pairs.index((i, j))
        oa = po.Tree.from_arrays(omra, *phis[i].download()[:2])
        ob = po.Tree.from_arrays(omra, *phis[j].download()[:2])
        t0 = time.perf_counter()
        orho = po.Tree(omra)
        po.multiply(prec / 10, orho, 1.0, oa, ob, -1, True, True)
        oV = po.Tree(omra)
        ost = po.apply(prec * 10, oV, oP, orho, abs_prec=True, prec_trees=[oa, ob] if i != j else [oa])
        cpu_s += time.perf_counter() - t0
        cpu_nodes += orho.nnodes + ost["out_nodes"]
        er, s1 = rel_vs_oracle(mra, rhos[k], orho)
        ev, s2 = rel_vs_oracle(mra, v64[k], oV)
        orac["rho"], orac["V"] = max(orac["rho"], er), max(orac["V"], ev)
        same = same and s1 and s2
    out["exchange_528"] = {
        "value": len(pairs) * world / (ms4 / 1e3), "unit": "pairs/s", "ms_per_step": ms4,
        "multiply_ms": mul_ms, "apply_ms": app_ms, "dtype": "df32 multiply + mixed apply",
        "multiply_host_split_ms": {"requests": sm["host_enum_ms"], "generation": sm["host_gen_ms"],
                                   "tasks": sm["host_items_ms"], "kernel_and_norms": sm["host_wait_ms"],
                                   "refinement": sm["host_refine_ms"], "compression": sm["gpu_post_ms"],
                                   "levels": sm["levels"], "launches": sm["launches"]},
        "nodes_per_s": (sm["out_nodes"] + sa["out_nodes"]) * world / (ms4 / 1e3),
        "input_nodes_total": int(sum(p.nnodes for p in phis)), "product_nodes": int(sum(r.nnodes for r in rhos)),
        "multiply_nodes_computed": sm["out_nodes"], "apply_output_nodes": sa["out_nodes"],
        "potential_err_vs_fp64_max": worst,
        "potential_err_unit": "|V_mixed - V_fp64| / max(|V_fp64|, 1): absolute precision",
        "rel_l2_vs_oracle_4_pairs": {"products": orac["rho"], "potentials_fp64": orac["V"],
                                     "pairs": sample, "node_sets_identical": same},
        "graph_captured": False,
        "cpu_baseline": {"value": len(sample) / cpu_s, "unit": "pairs/s", "cores": po.get_threads(), "kind": "port",
                         "sample": "pairs %s: multiply + FP64 apply each (%d nodes, %.1f s)" % (sample, cpu_nodes, cpu_s)}}
    # ---- adjoint check: Coulomb energy J = 1/2 <rho, P rho> of a 6-Gaussian density (k=9) ----
    prec = 1e-6
    rng = np.random.default_rng(SEED + 5)
    alphas = np.exp(rng.uniform(np.log(1.0), np.log(30.0), 6))
    centres = rng.uniform(-2, 2, (6, 3))
    terms = [((a / math.pi) ** 1.5, float(a), tuple(c), (0, 0, 0)) for a, c in zip(alphas, centres)]
    mra = mw.MultiResolutionAnalysis(9, device=device)
    rho = mw.project(prec, mw.FunctionTree(mra), terms, abs_prec=True)
    P = mw.PoissonOperator(mra, prec)
    V, AT = mw.FunctionTree(mra), mw.FunctionTree(mra)
    mw.copy_grid(V, rho)

    def fwd():
        return mw.apply_fixed(prec, V, P, rho, abs_prec=True)

    def adj():
        AT.clear()
        return mw.apply_adjoint(prec, AT, P, rho, rho)

    fwd_ms, stf = timed(fwd, steps)
    adj_ms, sta = timed(adj, steps)
    # <rho, A rho> = <A^T rho, rho>, and dJ/drho = (A + A^T) rho / 2 against the potential A rho
    lhs, rhs = mw.dot(rho, V), mw.dot(AT, rho)
    g = mw.FunctionTree(mra)
    mw.add(-1.0, g, [(0.5, V), (0.5, AT), (-1.0, V)])
    out["adjoint_k9"] = {
        "value": stf["out_nodes"] * world / (adj_ms / 1e3), "unit": "nodes/s (adjoint apply)",
        "ms_per_step": adj_ms, "forward_ms": fwd_ms, "dtype": "f64", "nodes": rho.nnodes,
        "items_forward": stf["items"], "items_adjoint": sta["items"],
        "dot_identity_rel_err": abs(lhs - rhs) / max(abs(lhs), 1e-300),
        "grad_minus_potential_rel_l2": g.norm() / max(V.norm(), 1e-300),
        "note": "fixed grid (the density's), absolute precision; the adjoint gathers by input node"}
    return out


def exchange_profile(mw, device, norb, reps):
    """The exchange-like workload of other_configs() on its first `norb` orbitals, `reps` times."""
    prec = 1e-5
    rng = np.random.default_rng(SEED)
    orbs = poly_orbitals(rng, 32, 0.5, 10.0)[:norb]
    mra = mw.MultiResolutionAnalysis(7, device=device)
    phis = []
    for t in orbs:
        f = mw.project(prec, mw.FunctionTree(mra), t, abs_prec=True)
        f.rescale(1.0 / f.norm())
        phis.append(f)
    pairs = [(i, j) for i in range(norb) for j in range(i, norb)]
    P = mw.PoissonOperator(mra, prec)
    pt = [[phis[i], phis[j]] if i != j else [phis[i]] for i, j in pairs]
    rhos = [mw.FunctionTree(mra) for _ in pairs]
    vmx = [mw.FunctionTree(mra) for _ in pairs]
    for _ in range(reps):
        for t in rhos + vmx:
            t.clear()
        sm = mw.multiply_batch(prec / 10, rhos, 1.0, [phis[i] for i, _ in pairs], [phis[j] for _, j in pairs],
                               abs_prec=True, use_max_norms=True)
        sa = mw.apply_batch(prec * 10, vmx, [P] * len(pairs), rhos, prec_trees=pt, abs_prec=True, precision="mixed")
    mra.synchronize()
    return {"pairs": len(pairs), "multiply": sm, "apply": sa}


def max_over_ranks(ms, device):
    """The slowest rank's time: every rank's timed region ends at a barrier, the job at its last rank."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(ms)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, t_max_ms):
    """Units processed by all ranks (each rank runs the same workload, weak scaling) per second."""
    return units_per_rank * world / (t_max_ms / 1e3)


def run(args):
    import torch

    import mrchem_gb300 as mw
    from mrchem_gb300 import build as mwbuild

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    mwbuild.build()
    mw.load_library()

    rng = np.random.default_rng(SEED)
    terms, mus = orbital_terms(rng)
    mra = mw.MultiResolutionAnalysis(ORDER, device=local)
    phis = []
    for t in terms:
        f = mw.project(PREC, mw.FunctionTree(mra), t, abs_prec=True)
        f.rescale(1.0 / f.norm())
        phis.append(f)
    t0 = time.perf_counter()
    ops = mw.HelmholtzOperator.batch(mra, mus, PREC)  # one operator per orbital, built together
    op_build_s = time.perf_counter() - t0
    in_nodes = [p.nnodes for p in phis]

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    def step(precision, outs):
        for o in outs:
            o.clear()
        return mw.apply_batch([PREC] * NORB, outs, ops, phis, abs_prec=True, precision=precision)

    outs = [mw.FunctionTree(mra) for _ in range(NORB)]

    def timed(precision, steps):
        """CUDA-event time per step of `steps` batched applies (after one untimed step)."""
        step(precision, outs)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record()
        for _ in range(steps):
            st_ = step(precision, outs)
        e1.record()
        barrier()
        return e0.elapsed_time(e1) / steps, st_

    if args.profile_exchange:
        # profiling mode: only the exchange-like workload on its first N orbitals (N(N+1)/2 pair
        # products and their Poisson applies), W + K times, for ncu captures of the multiply
        prof = exchange_profile(mw, local, args.profile_exchange, args.warmup + args.steps)
        print(json.dumps({"profile_exchange": True, **prof}))
        return
    if args.profile_mixed:
        # profiling mode: only the W + K mixed steps run (for a launch list of the headline step)
        for _ in range(args.warmup + args.steps):
            st_p = step("mixed", outs)
        barrier()
        print(json.dumps({"profile_mixed": True, "steps": args.warmup + args.steps, "stats": st_p}))
        return
    # plain FP64 GPU apply of the same batch: the baseline of the metric and the error reference
    fp64_ms, st64 = timed("fp64", args.fp64_steps)
    fp64_s = fp64_ms / 1e3
    ref = [mw.FunctionTree(mra) for _ in outs]
    for r, o in zip(ref, outs):
        mw.add(-1.0, r, [(1.0, o)])  # copy of the FP64 result

    def rel_err(a, r):
        """relative L2 norm of a - r, on the union grid (the grids may differ)"""
        d = mw.FunctionTree(mra)
        mw.add(-1.0, d, [(1.0, a), (-1.0, r)])
        return d.norm() / r.norm()

    near_ms, st_near = timed("mixed-near64", 1)
    near_err = max(rel_err(o, r) for o, r in zip(outs, ref))
    f32_ms, st_f32 = timed("mixed-fp32", 1)
    f32_err = max(rel_err(o, r) for o, r in zip(outs, ref))

    # launch settings (job groups, chunk sizes) picked for this batch by the autotuner; the timed
    # mixed steps below use them
    tuned = (mw.autotune_batch([PREC] * NORB, outs, ops, phis, abs_prec=True, precision="mixed", repeats=5)
             if args.autotune else None)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stats = []
    # the sampler starts before the warm-up steps (nvidia-smi takes a while to print its first
    # line); only the samples taken between the two marks are reported
    with ClockSampler() as clk:
        for _ in range(args.warmup):
            step("mixed", outs)
        barrier()
        # the interpreter's cyclic collector runs before the timed steps, not inside them
        gc.collect()
        gc.disable()
        clk.mark(True)
        start.record()
        for _ in range(args.steps):
            stats.append(step("mixed", outs))
        end.record()
        barrier()
        clk.mark(False)
        gc.enable()
    ms = start.elapsed_time(end) / args.steps
    nodes = stats[-1]["out_nodes"]
    errs = [rel_err(o, r) for o, r in zip(outs, ref)]
    t_max = max_over_ranks(ms, "cuda")
    value = whole_job_rate(nodes, world, t_max)

    # end-to-end through the C ABI: host input buffers -> device, apply, device -> host output.
    # One untimed step sizes the device trees and the host output buffers; every timed step then
    # uploads all inputs from host memory and downloads all outputs into those buffers.
    host_inputs = [p.download() for p in phis]
    e2e_phis = [mw.FunctionTree(mra) for _ in range(NORB)]
    h2d = sum(k.nbytes + c.nbytes for k, c, _ in host_inputs)
    host_outputs = [None] * NORB

    e2e_parts = {"upload_apply_download_ms": 0.0, "download_rest_ms": 0.0}

    def e2e_step():
        # mw_apply_batch_host: the inputs go up per job group, overlapped with the first groups'
        # levels, and each group's outputs go down into the pinned host buffers as soon as the
        # group is done
        t0 = time.perf_counter()
        for o in outs:
            o.clear()
        st_e = mw.apply_batch_host([PREC] * NORB, outs, ops, e2e_phis, host_inputs, abs_prec=True, precision="mixed",
                                   outputs=host_outputs if host_outputs[0] is not None else None)
        t1 = time.perf_counter()
        # outputs that did not go down with the apply (the first step, or a buffer too small)
        if not all(st_e.get("outputs_filled", [False])):
            host_outputs[:] = mw.download_batch(outs, outs=host_outputs if host_outputs[0] is not None else None)
        t2 = time.perf_counter()
        for k, v in zip(e2e_parts, (t1 - t0, t2 - t1)):
            e2e_parts[k] += v * 1e3
        return sum(a.nbytes for r in host_outputs for a in r)

    e2e_step()
    # the host buffers live in pinned memory (mw_pin_host), as a caller that keeps orbitals on the
    # host between steps would hold them: the copy engines then move them directly
    for _, c, _ in host_inputs:
        mw.pin_host(mra, c)
    for r in host_outputs:
        mw.pin_host(mra, r[1])
    # warm-up steps on the pinned buffers: the first call that overlaps the transfers with the job
    # groups sizes its staging and stream-ordered allocations
    e2e_each = []
    # the sampler starts before the warm-up steps, as for the device-resident loop: nvidia-smi's
    # start-up (its first samples come after a while) then overlaps them, not the timed steps
    with ClockSampler() as e2e_clk:
        for _ in range(max(3, args.warmup)):
            e2e_step()
        barrier()
        for k in e2e_parts:
            e2e_parts[k] = 0.0
        gc.collect()
        gc.disable()
        e2e_clk.mark(True)
        t0 = time.perf_counter()
        d2h = 0
        for _ in range(args.e2e_steps):
            ts = time.perf_counter()
            d2h = e2e_step()
            e2e_each.append((time.perf_counter() - ts) * 1e3)
        barrier()
        e2e_t1 = time.perf_counter()
        e2e_clk.mark(False)
    gc.enable()
    e2e_ms = max_over_ranks((e2e_t1 - t0) / args.e2e_steps * 1e3, "cuda")
    e2e_v = whole_job_rate(nodes, world, e2e_ms)

    st = stats[-1]
    # one step with the job groups not overlapped: its tier kernels run alone, so their
    # CUDA-event times are exclusive (the rooflines and the kernel split below use them)
    mra.set_overlap(False)
    serial_ms, st_ser = timed("mixed", 1)
    mra.set_overlap(True)
    # the same mixed step with the enumeration, screening and item lists on the host (OpenMP)
    # instead of the GPU; the item lists and results are identical
    mra.set_screening("host")
    host_scr_ms, st_hs = timed("mixed", 3)
    mra.set_screening("gpu")
    fp64_tf = mra.probe_fma_peak(True)
    fp32_tf = mra.probe_fma_peak(False)
    tf32_tf = mra.probe_mma_peak("tc05")          # tcgen05 TF32, M128 N256 K8: the device's dense rate
    tf32_n32_tf = mra.probe_mma_peak("tc05_n32")  # the same at the tier's own MMA shape, N = 32
    tf32_sync_tf = mra.probe_mma_peak("tf32")     # warp-level mma.sync m16n8k8 TF32, for comparison

    K = ORDER + 1
    # Work of one item (output node o, input node i, term t) in the cube formulation every tier
    # kernel uses: three passes, each contracting the (2K)^3 cube of the input block over one
    # dimension with a 2K x 2K operator block: 3 (2K)^4 multiply-adds = 6 (2K)^4 = 96 K^4 flops.
    work_item = 6.0 * (2 * K) ** 4
    # Every tier kernel sums the x passes of a row (consecutive items of a node with the same term,
    # ly and lz) and runs the y and z passes once per row: executed cube-pass work is 2 (2K)^4 flops
    # per item plus 4 (2K)^4 per row.
    pass_fl = 2.0 * (2 * K) ** 4
    # The tcgen05 tier issues its passes as M128 x N32 x K8 MMAs (mw_apply_tc05.cu's schedule):
    # ceil(4K^2/128) tiles in the x pass (per item), ceil(5K^2/128) in the y and z passes (per row),
    # ceil(ceil(2K/4)/2) k-steps each.
    ks = ((2 * K + 3) // 4 + 1) // 2
    tc_x_mmas = -(-4 * K * K // 128) * ks
    tc_yz_mmas = 2 * -(-5 * K * K // 128) * ks
    mma_fl = 2.0 * 128 * (32 if 3 * K > 16 else 16) * 8

    dram_per_item = DRAM_PER_ITEM
    tier_items = {"fp64": st_ser["items_fp64"], "fp32": st_ser["items_fp32"], "tf32": st_ser["items_tf32"],
                  "df32": st_ser["items_df"]}
    tier_rows = {"fp64": st_ser["rows_fp64"], "fp32": st_ser["rows_fp32"], "tf32": st_ser["rows_tf32"],
                 "df32": st_ser["rows_df"]}

    def roof(tier, ms, peak, kernel, bound, source, tc_mult=0):
        items, rows = tier_items[tier], tier_rows[tier]
        sec = ms / 1e3
        executed = items * pass_fl + rows * 2.0 * pass_fl
        ach = executed / sec / 1e12 if ms > 0 else 0.0
        out = {"bound": bound, "achieved": ach, "peak": peak, "unit": "TFLOP/s",
               "frac": ach / peak if peak else None,
               "work_unit": "cube-pass flops executed: 2 (2K)^4 per item (its x pass) + 4 (2K)^4 per row (the y "
                            "and z passes, once per run of a node's items with the same term, ly and lz)",
               "items": items, "rows": rows, "executed_flops": executed,
               "item_equivalent_rate": items * work_item / sec / 1e12 if ms > 0 else 0.0,
               "item_equivalent_unit": "6 (2K)^4 flops per item (three cube passes per item, as without rows)",
               "kernel": kernel, "kernel_ms_per_step": ms, "peak_source": source}
        if tc_mult:
            mmas = tc_mult * (items * tc_x_mmas + rows * tc_yz_mmas)
            iss = mmas * mma_fl / sec / 1e12 if ms > 0 else 0.0
            out.update({"issued_mmas_n32": mmas, "issued_achieved": iss, "issued_frac": iss / peak if peak else None})
        tr = dram_per_item.get(tier)
        out["traffic"] = tr * items if tr is not None else None
        out["traffic_unit"] = "DRAM bytes per step, all launches of the kernel" if tr is not None else None
        # the per-component-pair count (6 K^4 per surviving (ft, gt) pair, MRCPP's own unit), kept apart:
        # the cube passes share partial sums across pairs, so this rate can exceed the pipe's peak
        fl = st_ser["flops_" + ("df" if tier == "df32" else tier)]
        out["pair_unit_rate"] = fl / sec / 1e12 if ms > 0 else 0.0
        return out

    fma_src = "probed FMA throughput of this GPU (mw_probe_fma_peak); MEASURED_PEAKS.json holds no FP64/FP32 figure"
    mma_src = ("probed dense tcgen05.mma TF32 throughput of this GPU at M128 N256 K8 (mw_probe_mma_peak kind 2); "
               "MEASURED_PEAKS.json holds no TF32 figure")
    roofs = {
        "fp64": roof("fp64", st_ser["kernel_ms_fp64"], fp64_tf, "apply_kernel<double,10>", "fp64-pipe", fma_src),
        # the FP32-accuracy tier of the mixed step runs on the tensor cores as split TF32: per tile
        # and k-step A_hi * [B_hi B_lo] (width 64) and A_lo * B_hi (width 32), the issued work of
        # three N = 32 MMAs (hi*hi, hi*lo, lo*hi), 3 x the TF32 tier's
        "fp32": roof("fp32", st_ser["kernel_ms_fp32"], tf32_tf, "apply_tc05_kernel<10,1> (split TF32)", "tensor",
                     mma_src, tc_mult=3),
        "tf32": roof("tf32", st_ser["kernel_ms_tf32"], tf32_tf, "apply_tc05_kernel<10,0>", "tensor", mma_src,
                     tc_mult=1),
        # a double-FP32 multiply-add costs about 12 FP32 instructions in this kernel: its ceiling is the
        # FP32 FMA rate / 12 (multiply-adds), i.e. peak flops = FP32 FMA flops / 12
        "df32": roof("df32", st_ser["kernel_ms_df"], fp32_tf / 12.0, "apply_df_kernel<10>",
                     "fp32-pipe (double-FP32)", fma_src + "; divided by 12 FP32 instructions per double-FP32 "
                     "multiply-add"),
    }
    for t in ("tf32", "fp32"):
        roofs[t]["peak_tc05_n32"] = tf32_n32_tf
        roofs[t]["issued_frac_of_n32_rate"] = (roofs[t]["issued_achieved"] / tf32_n32_tf if tf32_n32_tf else None)
    roofs["tf32"]["peak_mma_sync_tf32"] = tf32_sync_tf
    dominant = max(roofs, key=lambda k: roofs[k]["kernel_ms_per_step"])
    line = {
        "metric": METRIC, "value": value, "unit": "nodes/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64+df32+f32+tf32", "data": "synthetic",
        "config": workload_config(),
        "workload_detail": {"tuned": tuned, "input_nodes": in_nodes, "input_nodes_total": int(sum(in_nodes)),
                            "output_nodes": nodes,
                            "l2": "inputs larger than L2 (%.2f GB of FP64 blocks against 129 MB of L2)"
                                  % (sum(in_nodes) * 8 * (ORDER + 1) ** 3 * 8 / 1e9),
                            "operator_terms": [o.nterms for o in ops], "operator_build_s": op_build_s},
        "fp64": {"value": st64["out_nodes"] * world / fp64_s, "unit": "nodes/s", "ms_per_step": fp64_ms,
                 "items": st64["items"], "kernel_ms_per_step": st64["kernel_ms"]},
        "mixed_near_fp64": {"value": st_near["out_nodes"] * world / (near_ms / 1e3), "unit": "nodes/s",
                            "ms_per_step": near_ms, "items_fp64": st_near["items_fp64"],
                            "items_fp32": st_near["items_fp32"], "rel_l2_vs_fp64_max": near_err,
                            "policy": "every |l|_inf <= 1 item kept in FP64"},
        "mixed_fp32": {"value": st_f32["out_nodes"] * world / (f32_ms / 1e3), "unit": "nodes/s",
                       "ms_per_step": f32_ms, "items_fp64": st_f32["items_fp64"], "items_fp32": st_f32["items_fp32"],
                       "rel_l2_vs_fp64_max": f32_err, "policy": "FP64 / FP32 tiers only (no tensor cores)"},
        "rel_l2_vs_fp64_max": max(errs),
        "items": {"total": st["items"], "fp64": st["items_fp64"], "fp32": st["items_fp32"], "tf32": st["items_tf32"],
                  "df32": st["items_df"]},
        "kernel_ms_per_step": st_ser["kernel_ms"], "host_ms_per_step": st["host_ms"],
        "host_breakdown_ms": {"enumerate": st["host_enum_ms"], "generate": st["host_gen_ms"], "items": st["host_items_ms"],
                              "launch": st["host_launch_ms"], "refine": st["host_refine_ms"],
                              "gpu_levels_span": st["gpu_levels_ms"], "gpu_post": st["gpu_post_ms"],
                              "wait_level": st["host_wait_ms"], "kernel_fp64": st_ser["kernel_ms_fp64"],
                              "kernel_fp32": st_ser["kernel_ms_fp32"], "kernel_tf32": st_ser["kernel_ms_tf32"],
                              "kernel_df32": st_ser["kernel_ms_df"],
                              "note": "host phases from the timed (overlapped) steps, with the screening on the "
                                      "GPU: enumerate = waiting for the walk's candidate counts, generate = "
                                      "queueing the generation, items = the tiers' node lists from the GPU's "
                                      "counts; exclusive kernel times from one step without overlap"},
        "no_overlap": {"value": st_ser["out_nodes"] * world / (serial_ms / 1e3), "unit": "nodes/s",
                       "ms_per_step": serial_ms, "policy": "job groups not pipelined (mw_ctx_set_overlap 0)"},
        "host_screening": {"value": st_hs["out_nodes"] * world / (host_scr_ms / 1e3), "unit": "nodes/s",
                           "ms_per_step": host_scr_ms,
                           "policy": "enumeration, screening and item lists on the host cores (mw_ctx_set_screening 0)"},
        "gpu_launches": int(st["launches"]),
        "e2e": {"value": e2e_v, "unit": "nodes/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "ms_per_step": e2e_ms, "ms_each_step": [round(x, 2) for x in e2e_each],
                # the mean above is the reported rate; the median shows a typical step beside it
                "ms_median_step": sorted(e2e_each)[len(e2e_each) // 2],
                "clocks": e2e_clk.summary(),
                "warmup": max(3, args.warmup), **{k: v / args.e2e_steps for k, v in e2e_parts.items()}},
        "roofline": dict(roofs[dominant], tier=dominant),
        "roofline_tiers": roofs,
        # the whole step against HBM: algorithmic bytes (FP64 blocks of every input and output
        # node, operator blocks used) over the step time; the step is compute-bound, so this
        # fraction is small by construction
        "hbm": {"achieved_gbs": st["bytes"] / (ms / 1e3) / 1e9,
                "peak_gbs": measured_peaks().get("hbm_gbs"),
                "frac": (st["bytes"] / (ms / 1e3) / 1e9 / measured_peaks()["hbm_gbs"])
                if measured_peaks().get("hbm_gbs") else None,
                "bytes_per_step": st["bytes"],
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy bandwidth)",
                "target_frac": 0.5, "target_met": False,
                "why": "compute-bound: each FP64 input block feeds hundreds of items, so the step's algorithmic "
                       "bytes take a fraction of a millisecond at HBM rate while its contractions take "
                       "milliseconds on the FP32, FP64 and tensor pipes"},
        "clocks": clk.summary(),
    }
    line["speedup_mixed_vs_fp64"] = (nodes / (ms / 1e3)) / (st64["out_nodes"] / fp64_s)
    if rank == 0 and not args.no_cpu:
        base, oracle_out = cpu_sample(terms, mus, args.cpu_s, keep=True)
        line["cpu_baseline"] = base
        # the GPU outputs of the sampled orbitals against the oracle's complete applies of them
        # (same orbitals, each side projecting its own input tree from the same Gaussians)
        vs, same = {"mixed": [], "fp64": []}, True
        for i, (ok, oc, _) in oracle_out.items():
            o_tree = mw.FunctionTree(mra).upload(ok, oc)
            vs["mixed"].append(rel_err(outs[i], o_tree))
            vs["fp64"].append(rel_err(ref[i], o_tree))
            same = same and np.array_equal(outs[i].download()[0], ok) and np.array_equal(ref[i].download()[0], ok)
        line["rel_l2_vs_oracle"] = {"mixed_max": max(vs["mixed"]), "fp64_max": max(vs["fp64"]),
                                    "orbitals": list(oracle_out), "node_sets_identical": bool(same)}
    if args.configs:
        line["configs"] = other_configs(mw, local, world, barrier, max(3, args.steps // 2))
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=30)
    ap.add_argument("--autotune", action=argparse.BooleanOptionalAction, default=True,
                    help="pick the batch's launch settings with mw_apply_batch_autotune before timing")
    ap.add_argument("--cpu-s", type=float, default=12.0,
                    help="seconds of oracle apply time for the cpu_baseline sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--configs", action=argparse.BooleanOptionalAction, default=True,
                    help="also time the other workloads (Poisson k=7, the batch at prec 1e-5 / 1e-7, exchange-like)")
    ap.add_argument("--orbitals", type=int, default=16)
    ap.add_argument("--fp64-steps", type=int, default=1)
    ap.add_argument("--profile-mixed", action="store_true")
    ap.add_argument("--profile-exchange", type=int, default=0, metavar="N",
                    help="run only the exchange-like workload on its first N orbitals (for ncu)")
    args = ap.parse_args()
    global NORB
    NORB = args.orbitals
    if args.impl == "reference":
        run_reference(args)
    else:
        run(args)


if __name__ == "__main__":
    main()
