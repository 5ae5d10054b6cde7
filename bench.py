"""Benchmark: explicit PD bond-updates/s on the 3D box-with-hole workload (C2).

Workload: 121x61x21-node (120x60x20 mm) Hex8 box, 8 mm central hole, 40x40
element PD zone through the thickness (31,584 families, 3.53 M directed bonds),
FP32 forces / FP64 integration, critical stretch 2e-3 +-5 % per bond, seeded
synthetic mesh.  One step = one explicit central-difference step of the whole
model (failure pass, PD + PD-boundary + FE force, update): one kernel launch.

  value   B * K / t over K device-resident steps (CUDA events on the model stream)
  e2e     same metric through pdx_explicit_step_host with pinned host buffers
          (u_n, u_n-1 in, u_n+1 out, copies inside the timed region)
  roofline  algorithmic bytes per step / mean step-kernel time vs measured HBM copy peak

--impl reference times the CPU restatement of the reference's path (the
oracle, all host threads) on the same model.  Under torchrun every rank runs an
independent replica on its own GPU (the path does not shard across GPUs).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "pdlsm-fem_mpi_gb300"))


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if not self.rows:
            # the timed region ended before nvidia-smi's first row: nothing is known
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def hold_clocks(index: int, advance, min_s: float = 1.0):
    """Clocks under the same step loop, run untimed right after the timed
    region for at least min_s seconds; used when the timed region was too short
    for nvidia-smi to sample it."""
    c = ClockSampler(index)
    c.start()
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < min_s:
        advance()
    out = c.stop()
    out["when"] = f"untimed hold of the same step loop for {time.perf_counter() - t0:.1f} s after the timed region"
    return out


TRAFFIC_PROFILE = {("c2", "MIXED"): "k_step_mixed_c2.md", ("c2", "FP64"): "k_step_fp64_c2.md",
                   ("c4", "MIXED"): "k_step_mixed_c4.md"}


def profile_traffic(workload: str, precision: str, alg_bytes: float):
    """DRAM bytes (read + write) per step-kernel launch from the committed ncu summary of this workload, scaled
    by algorithmic bytes when the capture ran a smaller case (C4: 64 of the 256 plates).  Returns (bytes, file)."""
    name = TRAFFIC_PROFILE.get((workload, precision))
    if not name:
        return None, None
    vals = {}
    try:
        with open(os.path.join(REPO, "profiles", name)) as f:
            for line in f:
                for key in ("traffic_bytes_per_launch", "algorithmic_bytes_per_launch"):
                    if line.startswith(key + ":"):
                        vals[key] = float(line.split(":", 1)[1])
    except (OSError, ValueError):
        return None, None
    if "traffic_bytes_per_launch" not in vals:
        return None, None
    t = vals["traffic_bytes_per_launch"]
    a = vals.get("algorithmic_bytes_per_launch")
    if a:
        t *= alg_bytes / a
    return int(round(t)), f"profiles/{name}"


def make_batch_workload(tmp: str, n_spec: int, nsteps: int, precision: str):
    import meshgen
    specs = meshgen.config_c4(n_spec=n_spec, nsteps=nsteps, precision=precision)
    return [meshgen.write_case(m, tmp, f"c4_{i:03d}", **kw) for i, (m, kw) in enumerate(specs)]


def cpu_sample_batch(cmds, target_s: float = 15.0, threads: int = 0):
    """Oracle on the first specimens of a batch, each from its initial state, until target_s of CPU work."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import orc
    import orc_setup
    bonds_steps, el, used = 0, 0.0, 0
    for c in cmds:
        host = orc_setup.load(c)      # the oracle's own set-up, not the library's
        o = orc.Oracle(host, nthreads=threads)
        t = time.perf_counter()
        o.explicit(nsteps=3)
        el += time.perf_counter() - t
        bonds_steps += host.info.n_bond * 4
        used += 1
        if el > target_s:
            break
    return bonds_steps / el, used, el, o_threads()


# The implicit legs (c3, c5) time whole solves; --steps is capped to this many samples.
IMPLICIT_MAX_STEPS = 5


def bench_implicit(args):
    """C5: implicit Newmark; solve time to a 1e-8 true FP64 residual per step for the learned two-level flexible CG,
    for block-Jacobi flexible CG (the plain method) and for block-Jacobi PCG in FP32 inside FP64 refinement (the
    mixed method), each from the same state after the training steps."""
    import meshgen
    import pdx
    tmp = tempfile.mkdtemp(prefix="pdx_bench_")
    steps = min(args.steps, IMPLICIT_MAX_STEPS)   # timed Newmark steps (each a whole solve)
    nsteps = args.train_steps + steps + 1
    if args.c5_size == "full":
        mesh, kw = meshgen.config_c5(nsteps=nsteps)
        cells = (25, 12, 5)
    elif args.c5_size == "medium":
        mesh, kw = meshgen.config_c5(nx=101, ny=51, nz=21, radius_h=5, nsteps=nsteps)
        cells = (12, 6, 3)
    else:
        mesh, kw = meshgen.config_c5(nx=61, ny=31, nz=13, radius_h=5, nsteps=nsteps)
        cells = (8, 4, 2)
    cmd = meshgen.write_case(mesh, tmp, "c5", **kw)
    res = {}
    for method in (4, 5, 3):
        with pdx.Model(cmd, device=0) as m:
            if method == 5:
                m.learned_setup(cells, hidden=128, seed=0, max_samples=(args.train_steps + args.probes) * 200)
            m.newmark_init()
            t0 = time.perf_counter()
            for _ in range(args.train_steps):
                m.newmark_step(4, collect=(method == 5))
            t_collect = time.perf_counter() - t0
            loss, t_train, pairs = None, 0.0, 0
            if method == 5:
                if args.probes:
                    t0 = time.perf_counter()
                    m.learned_probe(args.probes, seed=1)
                    t_collect += time.perf_counter() - t0
                pairs = m.learned_samples()
                t0 = time.perf_counter()
                loss = m.learned_train(epochs=100, lr=1e-3, seed=0)
                t_train = time.perf_counter() - t0
            sec, its, resid, refine, used = [], [], [], [], set()
            for _ in range(steps):
                i = m.newmark_step(method)
                sec.append(i.seconds)
                its.append(i.iterations)
                resid.append(i.rel_residual)
                refine.append(i.refinements)
                used.add(i.method_used)
            u = m.state()[0]
            res[method] = dict(sec=float(np.mean(sec)), its=float(np.mean(its)), resid=float(max(resid)), u=u,
                               loss=loss, t_train=t_train, t_collect=t_collect, pairs=pairs, n_eq=m.info.n_eq,
                               nnz=m.info.nnz, refine=float(np.mean(refine)), used=sorted(used))
    p, l, x = res[4], res[5], res[3]
    du = float(np.linalg.norm(l["u"] - p["u"]) / max(np.linalg.norm(p["u"]), 1e-300))
    dx = float(np.linalg.norm(x["u"] - p["u"]) / max(np.linalg.norm(p["u"]), 1e-300))
    line = {"metric": "implicit Newmark solve time to 1e-8 true residual (s per step)", "value": l["sec"],
            "unit": "s", "n_gpus": 1, "steps": steps, "warmup": args.train_steps, "ms_per_step": l["sec"] * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64 (network bf16/f32)",
            "data": "synthetic (seeded meshgen config_c5)",
            "config": {"workload": f"c5 ({args.c5_size}): Hex8 box, inclined penny crack, 5% PD zone, Newmark "
                                   f"beta 0.25 gamma 0.5, {p['n_eq']} equations, nnz {p['nnz']}",
                       "coarse_cells": cells, "hidden": 128, "train_steps": args.train_steps,
                       "probe_solves": args.probes},
            "plain": {"method": "block-Jacobi flexible CG", "s_per_step": p["sec"], "iterations": p["its"],
                      "max_rel_residual": p["resid"]},
            "learned": {"method": "flexible CG, block-Jacobi + learned coarse correction", "s_per_step": l["sec"],
                        "iterations": l["its"], "max_rel_residual": l["resid"], "training_pairs": l["pairs"],
                        "final_loss": l["loss"], "train_s": l["t_train"], "collect_s": l["t_collect"]},
            "speedup_vs_plain": p["sec"] / l["sec"] if l["sec"] > 0 else None,
            "u_rel_diff_learned_vs_plain": du,
            "mixed": {"method": "block-Jacobi PCG in FP32 (FP32 matrix copy) inside FP64 refinement",
                      "s_per_step": x["sec"], "iterations": x["its"], "refinement_steps": x["refine"],
                      "finished_by": x["used"], "max_rel_residual": x["resid"],
                      "speedup_vs_plain": p["sec"] / x["sec"] if x["sec"] > 0 else None,
                      "u_rel_diff_vs_plain": dx}}
    return line


def bench_quasi(args):
    """C3: the loaded quasi-static increment of the 401x401-node strip plate; device time of the solve to the 1e-8
    true FP64 residual for each Krylov method, beside a CPU direct solve (SuperLU through scipy, the stand-in for
    the reference's PARDISO) of the same system.  The reference's quasi-static rule puts the 1e-6 m top-edge pull
    on at the first increment and holds it (setVaryEssentialBC with load ratio 1), so increment 1 is unloaded and
    increment 2 carries the load; each timed sample re-initialises the model and times increment 2."""
    import meshgen
    import pdx
    tmp = tempfile.mkdtemp(prefix="pdx_bench_")
    mesh, kw = meshgen.config_c3(nsteps=2)
    cmd = meshgen.write_case(mesh, tmp, "c3", **kw)
    names = {0: "Jacobi PCG", 1: "block-Jacobi PCG", 2: "BiCGStab (Jacobi)", 3: "mixed FP32 PCG + FP64 refinement",
             6: "GMRES(30)", 7: "mixed FP32 BiCGStab + FP64 refinement",
             8: "BiCGStab, Jacobi + Galerkin coarse correction (20x20-cell lattice)"}
    res, u_end = {}, {}
    loaded = None
    # each sample is a whole solve (0.3 to 2 s): at most 5 timed after 1 untimed
    steps, warmup = min(args.steps, IMPLICIT_MAX_STEPS), min(args.warmup, 1)
    methods = [int(x) for x in args.c3_methods.split(",")]
    for method in methods:
        with pdx.Model(cmd, device=0, precision=0) as m:
            sec, its, resid, wall, used, refine, setup, setup_all = [], [], [], [], set(), [], [], []
            for rep in range(warmup + steps):
                m.quasi_init()
                i1 = m.quasi_step(method)
                setup_all.append(i1.setup_seconds)
                if loaded is None:
                    loaded = m.assemble(2, m.state()[0])
                t0 = time.perf_counter()
                i = m.quasi_step(method)
                if rep >= warmup:
                    wall.append(time.perf_counter() - t0)
                    sec.append(i.seconds)
                    its.append(i.iterations)
                    resid.append(i.rel_residual)
                    used.add(names.get(i.method_used, str(i.method_used)))
                    refine.append(i.refinements)
                    setup.append(i.setup_seconds)
                setup_all.append(i.setup_seconds)
            u_end[method] = m.state()[0]
            res[method] = dict(method=names[method], s_per_increment=float(np.mean(sec)),
                               increment_wall_s=float(np.mean(wall)), iterations=float(np.mean(its)),
                               max_rel_residual=float(max(resid)), finished_by=sorted(used))
            if method in (3, 7):
                res[method]["refinement_steps"] = float(np.mean(refine))
            if method == 8:
                # the coarse inverse is formed when the stiffness changes (the model's first solve here) and
                # reused while it does not: the loaded increment reassembles the same K as the unloaded one
                # (no bond broke), so the timed solves reuse it; the line also gives the time with it formed
                res[method]["coarse_setup_s"] = float(np.mean(setup))
                res[method]["coarse_setup_s_when_formed"] = float(max(setup_all))
                res[method]["s_per_increment_with_coarse_setup"] = float(np.mean(sec)) - float(np.mean(setup)) \
                    + float(max(setup_all))
            n_eq, nnz = m.info.n_eq, m.info.nnz
    ref = u_end[methods[0]]
    for k in res:
        res[k][f"u_rel_diff_vs_method_{methods[0]}"] = float(np.linalg.norm(u_end[k] - ref) / max(np.linalg.norm(ref), 1e-300))
    ia, ja, a, f = loaded
    cpu = None
    if not args.no_cpu_baseline:
        import scipy.sparse as sp
        import scipy.sparse.linalg as spla
        A = sp.csr_matrix((a, ja, ia), shape=(n_eq, n_eq))
        t0 = time.perf_counter()
        x_cpu = spla.spsolve(A.tocsc(), f)
        t_cpu = time.perf_counter() - t0
        x_gpu, info = pdx.solve_csr(ia, ja, a, f, method=1, rtol=1e-8, max_iter=20000)
        if not info.converged:
            x_gpu, info = pdx.solve_csr(ia, ja, a, f, method=2, rtol=1e-8, max_iter=20000)
        cpu = {"value": t_cpu, "unit": "s per increment (solve)", "cores": 1, "kind": "stand-in",
               "sample": "the loaded increment's K du = f solved once by SuperLU (scipy spsolve, 1 thread); "
                         "the reference factorises with PARDISO",
               "gpu_vs_direct_rel_diff": float(np.linalg.norm(x_gpu - x_cpu) / max(np.linalg.norm(x_cpu), 1e-300))}
    best = min(res.values(), key=lambda r: r["s_per_increment"])
    line = {"metric": "quasi-static solve time to 1e-8 true residual (s per loaded increment)",
            "value": best["s_per_increment"], "unit": "s", "n_gpus": 1, "steps": steps, "warmup": warmup,
            "ms_per_step": best["s_per_increment"] * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded meshgen config_c3)",
            "config": {"workload": f"c3: 2D quasi-static 401x401-node plate, PD band 30% of the width, 0.2 W "
                                   f"pre-crack, 1e-6 m top-edge pull, {n_eq} equations, nnz {nnz}",
                       "best_method": best["method"]},
            "methods": [res[k] for k in methods], "cpu_baseline": cpu}
    return line


def bench_fc1(args):
    """FC 1 crack growth (meshgen.fc1_bench_case): quasi-static increments of an n x n-node FE plate with an
    edge pre-crack (only the crack-cut elements PD at the start), K_Ic = 1 MPa m^0.5, top edge pulled 1e-6 m per
    load step.  Each
    increment assembles and solves K du = f (two-level BiCGStab, method 8, whose coarse inverse is re-formed
    after every PD-region growth), evaluates the crack tip's SIFs on the interaction-integral path and, from
    the first increment with Keq > K_Ic on, moves the tip, grows the PD region, breaks the bonds across the
    new segment and re-derives the device model.  One untimed run of 3 increments, then all increments timed
    on the host clock (the FC 1 pass and the rebuild are host work around the GPU kernels)."""
    import meshgen
    import pdx
    tmp = tempfile.mkdtemp(prefix="pdx_bench_")
    n = args.fc1_n
    nsteps = args.fc1_increments
    mesh, kw = meshgen.fc1_bench_case(n=n, nsteps=nsteps)
    cmd = meshgen.write_case(mesh, tmp, "fc1plate", **kw)
    method = 8
    with pdx.Model(cmd, device=0, precision=0) as m:
        m.quasi_init()
        for _ in range(3):
            m.quasi_step(method)
        m.quasi_init()
        wall, solve, moved, its, ki = [], [], [], [], []
        for _ in range(nsteps):
            t0 = time.perf_counter()
            i = m.quasi_step(method)
            wall.append(time.perf_counter() - t0)
            solve.append(i.seconds)
            its.append(i.iterations)
            moved.append(bool(m.crack_state()[0, 7]))
            ki.append(float(m.crack_state()[0, 4]))
        cs = m.crack_state()
        n_pde, n_fam, n_eq = m.array_len("pde_idx"), m.array_len("fam_off") - 1, m.info.n_eq
    wall, solve, moved = np.array(wall), np.array(solve), np.array(moved)
    grow = wall[moved] if moved.any() else np.zeros(1)
    load = wall[~moved] if (~moved).any() else np.zeros(1)
    return {"metric": "FC 1 quasi-static increment time (s per increment, crack-growth increments)",
            "value": float(grow.mean()), "unit": "s", "n_gpus": 1, "steps": nsteps, "warmup": 3,
            "ms_per_step": float(grow.mean()) * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded meshgen plate_edge_crack)",
            "config": {"workload": f"fc1: {n}x{n}-node FE plate, edge pre-crack to 0.41 W, FC 1 (mr 6, dcf 1), "
                                   f"K_Ic 1e6, top edge +1e-6 m per load step, {n_eq} equations",
                       "solve": "two-level BiCGStab (method 8) to 1e-10"},
            "growth_increments": int(moved.sum()), "load_increments": int((~moved).sum()),
            "s_per_load_increment": float(load.mean()), "s_per_growth_increment": float(grow.mean()),
            "solve_s_per_increment": float(solve.mean()), "iterations_per_increment": float(np.mean(its)),
            "host_and_rebuild_s_per_growth_increment": float((grow - solve[moved]).mean()) if moved.any() else None,
            "pd_elements_final": int(n_pde), "families_final": int(n_fam),
            "tip_final": [float(cs[0, 2]), float(cs[0, 3])], "keq_final": float(cs[0, 6]),
            "cpu_baseline": fc1_cpu_baseline(args, cmd, ki[1] if len(ki) > 1 else None)}


def fc1_cpu_baseline(args, cmd, ki_gpu):
    if args.no_cpu_baseline:
        return None
    t, ki = cpu_sample_fc1(cmd)
    return {"value": t, "unit": "s per increment", "cores": 1, "kind": "port",
            "sample": "the loaded increment (the first load step) by the oracle on one host thread: assembly, "
                      "K du = f by SuperLU (stand-in for the reference's PARDISO), node stresses, FC 1 SIFs",
            "ki_rel_diff_vs_gpu": None if ki_gpu is None else abs(ki - ki_gpu) / max(abs(ki), 1e-300)}


def cpu_sample_fc1(cmd: str):
    """The FC 1 plate's loaded increment (its first load step) on the host
    cores by the oracle: its own set-up and assembly (orc_setup, orc), K du = f
    by SuperLU (SciPy spsolve, one thread; the reference factorises with
    PARDISO), node stresses and the FC 1 evaluation (fc1_oracle).  Returns the
    seconds and the crack's KI."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import orc
    import orc_setup
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    from fc1_oracle import Fc1Oracle
    host = orc_setup.load(cmd, pattern=True)
    o = orc.Oracle(host)
    D = host.dim
    eq = host.array("eq")
    u = host.array("u0").copy()
    pres = eq < 0
    u[pres] += host.array("dtv").reshape(-1, 3)[:, :D].reshape(-1)[pres]
    t0 = time.perf_counter()
    ia, ja, a, f = o.assemble(u)
    n = len(ia) - 1
    du = spla.spsolve(sp.csr_matrix((a, ja, ia), shape=(n, n)).tocsc(), f)
    u[eq >= 0] += du[eq[eq >= 0]]
    cr = host.mesh.cracks[0]
    ev = Fc1Oracle(host, o, mr=host.cmd.mr, dcf=host.cmd.dcf)
    KI = ev.evaluate([cr[0][:2], cr[1][:2]], u.reshape(-1, D), host.array("bond_state0"))[0]
    return time.perf_counter() - t0, KI


# Steps per timed window.  Under the reference's failure model (PDLSM bond
# coefficients of the intact family kept while bonds break) C2 and C4 as
# configured run away after crack growth starts: C2 from about step 280 (the
# C restatement of the reference's loop does the same), C4's first plates from
# about step 225.  Steps past that point skip the force of most bonds and move
# NaN or infinite values, so they are not timed; C1 stays bounded over its
# 1,000 steps (and matches the reference's own run).
STEP_WINDOW = {"c1": 1001, "c2": 251, "c4": 201}
WINDOW_REASON = {
    "c1": "the configuration's 1,000 steps",
    "c2": "C2 stays bounded through step 250; its failure model runs away from about step 280",
    "c4": "every C4 plate stays bounded through step 200; the first ones run away from about step 225",
}


def make_workload(tmp: str, nsteps: int, precision: str):
    import meshgen
    mesh, kw = meshgen.config_c2(nsteps=nsteps, precision=precision)
    return meshgen.write_case(mesh, tmp, "c2", **kw)


def algorithmic_bytes(model) -> dict:
    """Unique bytes one step must move: per bond its member index, stored
    coefficients and state bit; per bond of a PD-boundary family its
    correction block; per node its displacements, velocity, mass and force
    state; per FE element its node ids."""
    info = model.info
    mixed = info.precision == 1
    cs = 4 if mixed else 8
    d = info.dim
    nsym = 3 if d == 2 else 6
    n_bond = info.n_bond
    fam_off = model.array("fam_off")
    pdbe_nodes = set(model.array("pdbe").reshape(-1, 4)[:, : (2 if d == 2 else 4)].ravel().tolist())
    fam_nodes = model.array("fam_members")[fam_off[:-1]]
    sizes = np.diff(fam_off) - 1
    corr_bonds = int(sum(int(s) for n, s in zip(fam_nodes, sizes) if n in pdbe_nodes))
    b_bond = 4 + nsym * cs + 1.0 / 8
    b_corr = d * d * cs
    b_node = 2 * d * 8 + 8 + d * 8 + (d * 4 if mixed else 0)
    b_elem = 4 * (4 if d == 2 else 8)
    total = n_bond * b_bond + corr_bonds * b_corr + info.n_node * b_node + info.n_fe * b_elem
    return {"bytes": total, "b_bond": b_bond, "b_corr": b_corr, "corr_bonds": corr_bonds, "b_node": b_node,
            "b_elem": b_elem}


def cpu_sample(cmd: str, target_s: float = 15.0, threads: int = 0, window: int = 1 << 30):
    """Oracle (CPU restatement of the reference path) on a bounded number of
    steps, in runs of at most `window` steps from the initial state (the
    window of the GPU timing).  Its set-up is the oracle's own
    (orc_setup), so this leg loads no product code."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import orc
    import orc_setup
    host = orc_setup.load(cmd)
    o = orc.Oracle(host, nthreads=threads)
    t = time.perf_counter()
    o.explicit(nsteps=1)
    one = (time.perf_counter() - t) / 2.0
    n = max(2, int(target_s / max(one, 1e-6)))
    el, done = 0.0, 0
    while done < n:
        k = min(n - done, window)
        t = time.perf_counter()
        o.explicit(nsteps=k - 1)
        el += time.perf_counter() - t
        done += k
    cores = o_threads()
    return host.info.n_bond * n / el, n, el, cores


def o_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def implicit_summary(args):
    """The implicit half of the metric beside the explicit line: C3's loaded
    quasi-static increment (every Krylov method, 3 timed solves each) and the
    C5 Newmark comparison of learned and plain flexible CG at the small size
    (61 x 31 x 13 nodes; the full size takes several minutes:
    --workload c5 --c5-size full)."""
    out = {}
    for name, extra in (("c3", {"steps": 3, "warmup": 1, "no_cpu_baseline": True}),
                        ("c5_small", {"steps": 3, "c5_size": "small"})):
        sub = argparse.Namespace(**vars(args))
        for k, v in extra.items():
            setattr(sub, k, v)
        try:
            r = bench_quasi(sub) if name == "c3" else bench_implicit(sub)
            keep = ("metric", "value", "unit", "config", "methods", "plain", "learned", "speedup_vs_plain", "mixed")
            out[name] = {k: r[k] for k in keep if k in r}
        except Exception as e:   # the explicit line stands without it
            out[name] = {"error": f"{type(e).__name__}: {e}"}
    return out


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="MIXED", choices=["MIXED", "FP64"])
    ap.add_argument("--e2e-steps", type=int, default=200)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-implicit", action="store_true",
                    help="c2: leave out the implicit sub-record (C3 increment, C5 small Newmark solves)")
    ap.add_argument("--lanes", type=int, default=-1,
                    help="lanes per PD family (-1: timed on the model by the library's autotuner, the default; "
                         "0: the library's fixed default)")
    ap.add_argument("--fe-lanes", type=int, default=-1, help="lanes per FE-only node (-1: timed, 0: fixed default)")
    ap.add_argument("--fc1-n", type=int, default=201, help="fc1: nodes per side of the plate")
    ap.add_argument("--fc1-increments", type=int, default=15, help="fc1: quasi-static increments timed")
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5", "fc1"],
                    help="c2: 3D box with hole (default); c1: 2D strip plate; c4: batch of uneven 2D plates in "
                         "one launch; c3: quasi-static increments, Krylov methods beside a CPU direct solve; "
                         "c5: implicit Newmark, learned vs plain preconditioner")
    ap.add_argument("--specimens", type=int, default=256, help="c4: number of specimens")
    ap.add_argument("--c3-methods", default="2,8,7,1,0,3",
                    help="c3: Krylov methods to time, comma separated (0 PCG, 1 block-Jacobi PCG, 2 BiCGStab, "
                         "3 mixed PCG + FP64 refinement, 6 GMRES, 7 mixed BiCGStab + FP64 refinement, 8 BiCGStab "
                         "with Jacobi + Galerkin coarse correction); the "
                         "first is the one the others' solutions are compared with")
    ap.add_argument("--c5-size", default="full", choices=["full", "medium", "small"],
                    help="c5: 201x101x41 nodes (full), 101x51x21 (medium) or 61x31x13 (small)")
    ap.add_argument("--train-steps", type=int, default=20, help="c5: Newmark steps that collect training pairs")
    ap.add_argument("--probes", type=int, default=60,
                    help="c5: random right-hand-side solves that add training pairs")
    args = ap.parse_args()
    if args.workload == "c5":
        print(json.dumps(bench_implicit(args)))
        return
    if args.workload == "c3":
        print(json.dumps(bench_quasi(args)))
        return
    if args.workload == "fc1":
        print(json.dumps(bench_fc1(args)))
        return
    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    tmp = tempfile.mkdtemp(prefix="pdx_bench_")
    nsteps_cmd = args.steps + args.warmup + 1
    if args.workload == "c2":
        cmd = make_workload(tmp, nsteps_cmd, args.precision)
        config = {"workload": "c2: 3D explicit box with hole, 121x61x21 nodes, Hex8 + PDLSM zone 40x40, "
                              "s0=2e-3+-5%",
                  "precision": args.precision, "inputs_vs_l2": "bond data streamed per step exceeds the 129 MB L2",
                  "step": "one central-difference step (failure + force + update)"}
    elif args.workload == "c1":
        import meshgen
        mesh, kw = meshgen.config_c1(nsteps=nsteps_cmd)
        kw["precision"] = args.precision
        cmd = meshgen.write_case(mesh, tmp, "c1", **kw)
        config = {"workload": "c1: 2D explicit 101x101-node plate, Q4 + central PD strip 41 nodes wide, 10 mm "
                              "edge pre-crack, s0=1e-3",
                  "precision": args.precision, "inputs_vs_l2": "L2-resident (about 2 MB per step)",
                  "step": "one central-difference step (failure + force + update)"}
    else:
        cmd = make_batch_workload(tmp, args.specimens, nsteps_cmd, args.precision)
        config = {"workload": f"c4: {args.specimens} 2D plates of 60x60..300x300 nodes (seeded), hole or edge "
                              "crack, PD band 10h, E 50-210 GPa, s0 5e-4..3e-3, one launch per step",
                  "precision": args.precision, "inputs_vs_l2": "per-step node and bond data exceed the 129 MB L2",
                  "step": "one central-difference step of every specimen (failure + force + update)"}
    if args.impl == "reference":
        if rank != 0:
            return
        rate, n, el, cores = cpu_sample(cmd, target_s=20.0, window=STEP_WINDOW[args.workload]) \
            if args.workload != "c4" else \
            cpu_sample_batch(cmd, target_s=20.0)
        line = {"metric": "explicit PD bond-updates/s", "value": rate, "unit": "bond-updates/s", "n_gpus": args.gpus,
                "steps": n, "warmup": 0, "ms_per_step": el / n * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config, "impl": "reference",
                "cpu_baseline": {"value": rate, "unit": "bond-updates/s", "cores": cores, "kind": "port",
                                 "sample": (f"{n} explicit steps of the full {args.workload.upper()} model on "
                                            f"{cores} host threads, in runs of at most "
                                            f"{STEP_WINDOW[args.workload]} steps from the initial state"
                                            if args.workload != "c4" else
                                            f"4 explicit steps of each of the first {n} specimens on {cores} "
                                            "host threads")},
                "e2e": {"value": rate, "unit": "bond-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    import pdx
    prec = 1 if args.precision == "MIXED" else 0
    if args.workload != "c4":
        model = pdx.Model(cmd, device=local, precision=prec, lanes=args.lanes, fe_lanes=args.fe_lanes)
    else:
        model = pdx.Model.batch(cmd, device=local, precision=prec, lanes=args.lanes, fe_lanes=args.fe_lanes)
    info = model.info
    config["lanes"] = {"per_family": info.lanes, "per_fe_node": info.fe_lanes,
                       "chosen": "timed on the model (pdx_options lanes = -1)" if args.lanes < 0 or args.fe_lanes < 0
                       else "fixed"}
    alg = algorithmic_bytes(model)
    # warm-up steps (step 0 included), then the timed region in windows that
    # restart from the initial state, each within the steps the model keeps
    # bounded (STEP_WINDOW); the re-initialisation between windows is untimed
    window = STEP_WINDOW[args.workload]
    model.explicit_init()
    model.explicit_advance(args.warmup)
    clocks = ClockSampler(local)
    clocks.start()
    ms, left, n_windows = 0.0, args.steps, 0
    while left > 0:
        n = min(window - 1, left)
        model.explicit_init()
        model.explicit_advance(1)        # step 0 (u1 = u0 + dt^2/2 a0), untimed
        if dist:
            dist.barrier()
        ms += model.explicit_advance_timed(n)
        left -= n
        n_windows += 1
    clk = clocks.stop()
    if clk.get("samples", 0) < 3:
        model.explicit_init()
        clk["hold"] = hold_clocks(local, lambda: (model.explicit_init(), model.explicit_advance(window - 1)))
    config["timed_windows"] = (f"{n_windows} window(s) of up to {window - 1} steps after step 0, each from the "
                               f"initial state: {WINDOW_REASON[args.workload]}")
    t_s = ms * 1e-3
    if dist:
        import torch
        t = torch.tensor([t_s], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_s = float(t.item())
    value = info.n_bond * args.steps * ws / t_s
    # end to end through the host-buffer entry point
    eq = model.array("eq")
    act = eq >= 0
    u0 = model.array("u0")
    import ctypes
    def pinned(n):
        try:
            import torch
            return torch.zeros(n, dtype=torch.float64, pin_memory=True).numpy()
        except Exception:
            return np.zeros(n)
    un, unm1, out = pinned(info.n_eq), pinned(info.n_eq), pinned(info.n_eq)
    # the three pinned buffers rotate roles (u_n+1 of one step is u_n of the
    # next); the same bounded windows as the device-resident timing
    t_e2e, left = 0.0, args.e2e_steps
    while left > 0:
        n = min(window - 4, left)
        un[:] = 0.0
        un[eq[act]] = u0[act]
        unm1[:] = un
        model.explicit_init()
        for _ in range(3):
            model.explicit_step_host(un, unm1, out)
            un, unm1, out = out, un, unm1
        t0 = time.perf_counter()
        for _ in range(n):
            model.explicit_step_host(un, unm1, out)
            un, unm1, out = out, un, unm1
        t_e2e += time.perf_counter() - t0
        left -= n
    e2e = info.n_bond * args.e2e_steps / t_e2e
    peak, kind = measured_peaks()
    achieved = alg["bytes"] / (t_s / args.steps) / 1e9
    traffic, traffic_src = profile_traffic(args.workload, args.precision, alg["bytes"])
    line = {"metric": "explicit PD bond-updates/s", "value": value, "unit": "bond-updates/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 forces / f64 state" if args.precision == "MIXED"
            else "f64", "data": f"synthetic (seeded meshgen config_{args.workload})", "config": config,
            "e2e": {"value": e2e, "unit": "bond-updates/s", "h2d_bytes_per_step": 2 * info.n_eq * 8,
                    "d2h_bytes_per_step": info.n_eq * 8, "steps": args.e2e_steps},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": traffic,
                         "traffic_unit": f"bytes per launch (ncu, {traffic_src}; scaled by algorithmic bytes to "
                                         f"this workload)" if traffic_src else None, "peak_kind": kind,
                         "algorithmic_bytes_per_step": alg["bytes"], "kernel": "k_step"},
            "gpu_launches": args.steps, "clocks": clk,
            "model": {"n_node": info.n_node, "n_fam": info.n_fam, "n_bond": info.n_bond, "n_eq": info.n_eq,
                      "n_fe": info.n_fe, "lanes": info.lanes, "fe_lanes": info.fe_lanes}}
    if rank == 0 and not args.no_cpu_baseline:
        if args.workload != "c4":
            rate, n, el, cores = cpu_sample(cmd, target_s=15.0, window=STEP_WINDOW[args.workload])
            sample = f"{n} explicit steps of the full model (FP64 oracle) on {cores} threads"
        else:
            rate, n, el, cores = cpu_sample_batch(cmd, target_s=15.0)
            sample = f"4 explicit steps of each of the first {n} specimens (FP64 oracle) on {cores} threads"
        line["cpu_baseline"] = {"value": rate, "unit": "bond-updates/s", "cores": cores, "kind": "port",
                                "sample": sample}
    model.close()
    if rank == 0 and ws == 1 and args.workload == "c2" and not args.no_implicit:
        line["implicit"] = implicit_summary(args)
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
