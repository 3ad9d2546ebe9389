"""Benchmark: FP64 DOF·stage-updates/s of the DGSEM residual + SSP-RK3 on one GB300.

Workload (3D compressible Euler Taylor-Green vortex, Mach 0.1, ρ0 = 1, p0 = 1/(γM²), periodic
[0, 2π]³, split-form flux differencing with the Chandrashekar two-point flux, HLLC interface
flux, SSP-RK3):  mesh A = 32³ elements at p = 3, mesh B = 16³ elements at p = 7
(2,097,152 nodes each).  One bench step = one SSP-RK3 step of A and one of B.
A DOF is a solution node (all 5 variables); one DOF·stage-update advances one node through
one RK stage (residual + stage combination).

  value   device-resident throughput (states already in HBM), CUDA events on the launching
          stream, K steps between synchronised barriers, max over ranks
  e2e     the same metric through the public API with pinned host buffers: every step copies
          the state host->device, advances it and copies it back
  --impl reference   the CPU oracle (the C++ restatement of Flou's residual), all host
          threads, on a bounded sample mesh of the same configuration

Under torchrun (N > 1) every rank runs its own replica of the workload (the path has no
exchange step); value = total DOF·stage-updates of all ranks / max time.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "flou.jl_gb300"))

import numpy as np

METRIC = "FP64 DOF·stage-updates/s (residual + SSP-RK3 stage), 3D Euler TGV split-form"
UNIT = "DOF·stage-updates/s"
NV = 5
BYTES_PER_DOF_STAGE = (8.0 / 3.0) * NV * 8   # compulsory state traffic, fused SSP-RK3


def replica_throughput(local_ms, local_units, dist=None, device=None):
    """Replicas of the workload, one per rank, no data exchange: the job's throughput is the
    units all ranks processed divided by the slowest rank's time.  Returns (value, max_ms)."""
    if dist is None:
        return local_units / (local_ms * 1e-3), local_ms
    import torch
    t = torch.tensor([local_ms, local_units], dtype=torch.float64, device=device)
    mx = t[:1].clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    tot = t[1:].clone()
    dist.all_reduce(tot, op=dist.ReduceOp.SUM)
    return float(tot) / (float(mx) * 1e-3), float(mx)


# Fixed dt of the Taylor-Green meshes: TGV_CFL x get_max_dt(U0, 1).  At p = 7 a CFL of 0.2 in
# get_max_dt's definition (mean node spacing) is unstable with SSP-RK3: the 16^3 p=7 mesh, and
# the oracle on 4^3 p=7, lose positivity within 50-100 steps; 0.15 is stable over 100 steps.
TGV_CFL = 0.15


def make_tgv(nel, n, mach=0.1):
    import flou_cuda as F
    eq = F.EulerEquation(3, 1.4)
    mesh = F.CartesianMesh((0.0, 0.0, 0.0), (2 * math.pi,) * 3, (nel,) * 3)
    F.apply_periodicBCs(mesh, ("1", "2"), ("3", "4"), ("5", "6"))
    b = F.LagrangeBasis("GLL", n)
    std = F.StdHex(b, F.DGSEMrec(b), eq.nvariables)
    disc = F.MultielementDisc(mesh, std, eq, F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC()), {})
    Q0 = np.asfortranarray(F.initial.taylor_green(eq, disc.coords, mach=mach))
    return disc, Q0


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms in the background."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.th = threading.Thread(target=self._read, daemon=True)
        self.th.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.th.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "", 1).isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "", 1).isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) >= 9 for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def load_profile_summary():
    """Per-DOF DRAM traffic and executed FP64 operations of the element kernels, from the
    committed ncu summary (profiles/)."""
    p = os.path.join(ROOT, "profiles", "tgv3d_split_elem_kernel.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


WORKLOAD = "tgv3d_M0.1_split_chandrashekar_hllc_ssprk3: 32^3 p=3 + 16^3 p=7"
FULL_NDOFS = 32 ** 3 * 4 ** 3 + 16 ** 3 * 8 ** 3   # 4,194,304 nodes


def cpu_oracle_rate(steps, warmup, threads):
    """The CPU oracle on the workload's own meshes: one SSP-RK3 step of the 32³ p=3 mesh and one
    of the 16³ p=7 mesh (2,097,152 nodes each) per step, every step from the initial state.
    Returns (rate, seconds, ndofs)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_ref
    from cases import oracle_for
    L = oracle_ref.lib()
    L.oracle_set_threads(threads)
    samples = []
    for nel, n in ((32, 4), (16, 8)):
        disc, Q0 = make_tgv(nel, n)
        o = oracle_for(disc)
        dt = TGV_CFL * o.max_dt(Q0, 1.0, disc.std.omega)
        samples.append((o, Q0, dt, disc.ndofs))
    for _ in range(warmup):
        for o, Q0, dt, _n in samples:
            o.ssprk3(Q0, dt, 1)
    t0 = time.perf_counter()
    for _ in range(steps):
        for o, Q0, dt, _n in samples:
            o.ssprk3(Q0, dt, 1)
    sec = time.perf_counter() - t0
    ndofs = sum(s[3] for s in samples)
    return ndofs * 3 * steps / sec, sec, ndofs


def workload_config(world):
    """The `config` object of both arms (the same workload, the same keys)."""
    return {"workload": WORKLOAD, "ndofs_per_gpu": FULL_NDOFS, "parallelism": "replicas" if world > 1 else "single",
            "l2": "inputs larger than L2: each stage streams ~250 MB per mesh (L2 129 MB)",
            "schedule": "one stream per mesh, steps pipelined per mesh (value and e2e)"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    steps = max(args.steps, 1)
    rate, sec, ndofs = cpu_oracle_rate(steps, args.warmup, threads)
    sample = ("%d SSP-RK3 steps of the workload's two meshes (32^3 p=3 and 16^3 p=7, %d nodes) after %d warm-up "
              "steps, each from the initial state; the C++ restatement of Flou's residual and SSP-RK3 (Flou's Julia "
              "path cannot run here: no julia), OpenMP over elements and faces" % (steps, ndofs, args.warmup))
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sec / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(1),
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def make_batched(count=256, seed=2026, nmin=8, nmax=64):
    """The batched configuration: `count` independent 2D Euler instances on [-5,5]², n×n
    elements with n ~ U{nmin..nmax}, p ~ U{2..7}, periodic or slip walls (50/50), isentropic
    vortex of strength U(1,6) plus a Gaussian density bump of amplitude U(0,0.1), Rusanov flux,
    strong form, SSP-RK3 with a fixed per-instance dt = get_max_dt(U0, cfl=0.2) (at 0.3, 67 of the
    256 instances -- p = 6, 7 -- become unstable within 60 steps; all are stable at 0.2)."""
    import flou_cuda as F
    rng = np.random.default_rng(seed)
    eq = F.EulerEquation(2, 1.4)
    out = []
    for k in range(count):
        ne = int(rng.integers(nmin, nmax + 1))
        n = int(rng.integers(3, 9))
        walls = bool(rng.integers(0, 2))
        mesh = F.CartesianMesh((-5.0, -5.0), (5.0, 5.0), (ne, ne))
        if walls:
            bcs = {str(b): F.EulerSlipBC() for b in range(1, 5)}
        else:
            F.apply_periodicBCs(mesh, ("1", "2"), ("3", "4"))
            bcs = {}
        b = F.LagrangeBasis("GLL", n)
        std = F.StdQuad(b, F.DGSEMrec(b), eq.nvariables)
        disc = F.MultielementDisc(mesh, std, eq, F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)), bcs)
        Q0 = F.initial.vortex_bump(eq, disc.coords, rng.uniform(-2, 2, 2), rng.uniform(1, 6), rng.uniform(0, 0.1),
                                   uinf=(0.0, 0.0) if walls else (1.0, 1.0), period=None if walls else (10.0, 10.0))
        out.append((disc, np.asfortranarray(Q0)))
    return out


def bench_batched(steps, warmup, count=256):
    """Batched (one persistent launch per stage for all instances) against the same instances
    stepped one by one with the plain kernels (one flou_step call per instance)."""
    import torch
    import flou_cuda as F
    insts = make_batched(count)
    stream = torch.cuda.current_stream()
    discs = [d for d, _ in insts]
    Qs = [torch.from_numpy(np.ascontiguousarray(Q.T)).cuda() for _, Q in insts]
    dts = [0.2 * d.ctx.max_dt(q, 1.0) for d, q in zip(discs, Qs)]
    ndofs = sum(d.ndofs for d in discs)
    batch = F.Batch(discs, Qs, dts)
    batch.set_stream(stream.cuda_stream)
    choice = batch.autotune()
    for _ in range(warmup):
        batch.step(1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    batch.step(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_b = e0.elapsed_time(e1)
    # one by one, from the same initial states: each instance advanced `steps` steps with its own
    # graph, then the next
    for q, (_, Q) in zip(Qs, insts):
        q.copy_(torch.from_numpy(np.ascontiguousarray(Q.T)))
    for d in discs:
        d.ctx.set_stream(stream.cuda_stream)
    for d, q, dt in zip(discs, Qs, dts):
        d.ctx.step(q, dt, warmup)
    torch.cuda.synchronize()
    e0.record(stream)
    for d, q, dt in zip(discs, Qs, dts):
        d.ctx.step(q, dt, steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_s = e0.elapsed_time(e1)
    for d in discs:
        d.ctx.set_stream(0)
    # Where the serial loop's time goes.  The throughput floor: the plain face and element
    # kernels of each order timed (CUDA events, the three stage modes averaged) on one large
    # periodic mesh of that order (~1.5 M nodes, many waves: full occupancy, no tail), giving the
    # cost per node and stage when nothing but the kernels' own work is left; every instance
    # priced at its order's rate is the time the same tile code needs with no launch, latency
    # or tail overhead -- what any batching of these kernels can at best reach.
    orders = sorted({d.std.n for d in discs})
    per_node = {}
    by_order = {}
    eq = discs[0].equation
    for n in orders:
        ne = max(8, int(round(math.sqrt(1.5e6) / n)))
        mesh = F.CartesianMesh((-5.0, -5.0), (5.0, 5.0), (ne, ne))
        F.apply_periodicBCs(mesh, ("1", "2"), ("3", "4"))
        b = F.LagrangeBasis("GLL", n)
        big = F.MultielementDisc(mesh, F.StdQuad(b, F.DGSEMrec(b), eq.nvariables), eq,
                                 F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)), {})
        qb = torch.from_numpy(np.ascontiguousarray(
            F.initial.vortex_bump(eq, big.coords, (0.3, -0.2), 3.0, 0.05, period=(10.0, 10.0)).T)).cuda()
        fms, ems = big.ctx.time_kernels(qb, nrep=3)
        per_node[n] = (fms + ems) / big.ndofs
        ks = [k for k, d in enumerate(discs) if d.std.n == n]
        by_order["p%d" % (n - 1)] = {
            "instances": len(ks), "ndofs": sum(discs[k].ndofs for k in ks),
            "floor_ms_per_step": 3 * per_node[n] * sum(discs[k].ndofs for k in ks),
            "rate_mesh_ndofs": big.ndofs, "ns_per_node_stage": 1e6 * per_node[n]}
        del big, qb
    floor_ms = 3 * sum(per_node[d.std.n] * d.ndofs for d in discs)
    vb = ndofs * 3 * steps / (ms_b * 1e-3)
    vs = ndofs * 3 * steps / (ms_s * 1e-3)
    return {"value": vb, "unit": UNIT, "serial_value": vs, "speedup_vs_serial": vb / vs, "instances": count,
            "ndofs": ndofs, "ms_per_step": ms_b / steps, "serial_ms_per_step": ms_s / steps, "autotune": choice,
            "throughput_floor_ms_per_step": floor_ms, "batched_over_floor": (ms_b / steps) / floor_ms,
            "speedup_bound_at_floor": (ms_s / steps) / floor_ms, "by_order": by_order,
            "gpu_launches_per_step": 3, "serial_gpu_launches_per_step": 6 * count,
            "workload": "256 x 2D Euler, n~U{8..64}^2 elements, p~U{2..7}, periodic/slip walls, vortex+bump, "
                        "Rusanov, strong form, SSP-RK3"}


def bench_adjoint(nsteps=400, nsnap=20, ndirs=32, seed=404):
    """The adjoint configuration: 2D Euler, 64x64 elements, p=4, periodic [-5,5]², 400 SSP-RK3
    steps at CFL 0.4 (0.5 in get_max_dt's definition is unstable with SSP-RK3 at p=4, also on the
    CPU oracle), J = 1/2 Σ w (ρ(T) - ρt)² with quadrature weights w = Jω and ρt the density of
    a perturbed vortex carried to T; gradients with respect to U0 and the per-element dissipation
    scales c (at c = 1) with 20 snapshots, checked against central differences (h = 1e-6) along
    `ndirs` random directions."""
    import torch
    import flou_cuda as F
    rng = np.random.default_rng(seed)
    eq = F.EulerEquation(2, 1.4)
    mesh = F.CartesianMesh((-5.0, -5.0), (5.0, 5.0), (64, 64))
    F.apply_periodicBCs(mesh, ("1", "2"), ("3", "4"))
    b = F.LagrangeBasis("GLL", 5)
    disc = F.MultielementDisc(mesh, F.StdQuad(b, F.DGSEMrec(b), 4), eq, F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)))
    ctx = disc.ctx
    center = rng.uniform(-1, 1, 2)
    Q0 = np.asfortranarray(F.initial.isentropic_vortex(eq, disc.coords, center, beta=5.0, period=(10.0, 10.0)))
    c = np.ones(mesh.nelements)
    ctx.set_dissipation(c)
    Qd = torch.from_numpy(np.ascontiguousarray(Q0.T)).cuda()
    dt = 0.4 * ctx.max_dt(Qd, 1.0)
    T = nsteps * dt
    tgt = F.initial.isentropic_vortex(eq, disc.coords, center + T + rng.normal(0, 0.1, 2), beta=5.0 + rng.normal(0, 0.2),
                                      period=(10.0, 10.0))
    rho_t = torch.from_numpy(np.ascontiguousarray(tgt[:, 0])).cuda()
    w = torch.from_numpy(np.tile(disc.std.omega, mesh.nelements) * disc.J).cuda()
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def forward(Q, cc=None):
        if cc is not None:
            ctx.set_dissipation(cc)
        q = Q.clone()
        ctx.step(q, dt, nsteps)
        r = q[0] - rho_t
        return float(0.5 * torch.sum(w * r * r))

    forward(Qd)   # warm-up (graph capture)
    torch.cuda.synchronize()
    ev[0].record(stream)
    J0 = forward(Qd)
    ev[1].record(stream)
    torch.cuda.synchronize()
    fwd_ms = ev[0].elapsed_time(ev[1])
    g = torch.empty_like(Qd)
    gc = torch.empty(mesh.nelements, dtype=torch.float64, device="cuda")
    res = {}
    for tag, ns in (("", nsnap), ("_store_all", nsteps - 1)):
        ctx.adjoint_solve(Qd, dt, nsteps, ns, rho_t, w, g, gc)   # warm-up
        torch.cuda.synchronize()
        ev[0].record(stream)
        J, nfwd = ctx.adjoint_solve(Qd, dt, nsteps, ns, rho_t, w, g, gc)
        ev[1].record(stream)
        torch.cuda.synchronize()
        res["adjoint_ms" + tag] = ev[0].elapsed_time(ev[1])
        res["recomputed_forward_steps" + tag] = nfwd
        res["snapshots" + tag] = ns
    gh, gch = g.cpu().numpy(), gc.cpu().numpy()
    h = 1e-6
    errs = []
    for k in range(ndirs):
        dQ = torch.from_numpy(rng.standard_normal(Q0.shape[::-1])).cuda()
        dc = rng.standard_normal(c.shape)
        fd = (forward(Qd + h * dQ, c + h * dc) - forward(Qd - h * dQ, c - h * dc)) / (2 * h)
        ours = float(np.sum(gh * dQ.cpu().numpy()) + np.sum(gch * dc))
        errs.append(abs(ours - fd) / abs(fd))
    ctx.set_dissipation(c)
    ctx.set_stream(0)
    res.update({"forward_ms": fwd_ms, "ratio": res["adjoint_ms"] / fwd_ms,
                "ratio_store_all": res["adjoint_ms_store_all"] / fwd_ms, "J": J0, "steps": nsteps,
                "ndofs": disc.ndofs, "fd_directions": ndirs, "fd_h": h, "fd_max_rel_err": max(errs),
                "fd_median_rel_err": float(np.median(errs)),
                "workload": "2D Euler 64x64 p=4 periodic vortex, 400 SSP-RK3 steps, dJ/dU0 and dJ/dc, 20 snapshots"})
    return res


def bench_curvilinear(steps, warmup, stream, kern_cart):
    """The general-geometry kernels on mesh A's size: a periodic-free [0, 2π]³ box of 32³
    straight-sided hexahedra with interior nodes displaced by 10% of a cell and every element's
    local numbering rotated at random (all master2slave orientations), p = 3, TGV Mach 0.1,
    split form with the Chandrashekar flux and HLLC, outflow boundaries."""
    import torch
    import flou_cuda as F
    t0 = time.perf_counter()
    mesh = F.perturbed_box(3, 32, (0.0,) * 3, (2 * math.pi,) * 3, amp=0.1, seed=1)
    eq = F.EulerEquation(3, 1.4)
    b = F.LagrangeBasis("GLL", 4)
    disc = F.MultielementDisc(mesh, F.StdHex(b, F.DGSEMrec(b), 5), eq,
                              F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC()),
                              {k: F.EulerOutflowBC() for k in mesh.bdnames})
    Q0 = np.asfortranarray(F.initial.taylor_green(eq, disc.coords, mach=0.1))
    setup_s = time.perf_counter() - t0
    ctx = disc.ctx
    ctx.set_stream(stream.cuda_stream)
    q = torch.from_numpy(np.ascontiguousarray(Q0.T)).cuda()
    dt = 0.2 * ctx.max_dt(q, 1.0)
    ctx.step(q, dt, warmup)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    ctx.step(q, dt, steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    fms, ems = ctx.time_kernels(q, nrep=3)
    ctx.set_stream(0)
    units = disc.ndofs * 3
    return {"value": units / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "face_ms": fms, "elem_ms": ems,
            "ndofs": disc.ndofs, "cartesian_face_ms": kern_cart["face_ms"], "cartesian_elem_ms": kern_cart["elem_ms"],
            "elem_cost_vs_cartesian": ems / kern_cart["elem_ms"], "face_cost_vs_cartesian": fms / kern_cart["face_ms"],
            "orientations": sorted(set(int(o) for o in mesh.orientation)), "setup_s": setup_s,
            "workload": "32^3 perturbed (10%) rotated hex, p=3, TGV M0.1, split Chandrashekar + HLLC, outflow"}


def make_adjoint_batch(count=64, seed=505, mmin=8, mmax=24):
    """The batched-adjoint configuration: `count` periodic [0, 2π]³ hex meshes of m³ elements,
    m ~ U{8..24}, p ~ U{3, 4, 5}, Taylor-Green vortex at Mach ~ U(0.05, 0.3) (plus a 1e-3 smooth
    perturbation), split form with the
    Chandrashekar two-point flux and the LxF(ChandrasekharAverage) interface flux (the interface
    flux the adjoint differentiates), per-element dissipation scale c = 1."""
    import flou_cuda as F
    rng = np.random.default_rng(seed)
    prng = np.random.default_rng(seed + 1)   # perturbations: the instance draws stay those of `seed`
    eq = F.EulerEquation(3, 1.4)
    out = []
    for _ in range(count):
        m = int(rng.integers(mmin, mmax + 1))
        p = int(rng.integers(3, 6))
        mach = float(rng.uniform(0.05, 0.3))
        mesh = F.CartesianMesh((0.0, 0.0, 0.0), (2 * math.pi,) * 3, (m,) * 3)
        F.apply_periodicBCs(mesh, ("1", "2"), ("3", "4"), ("5", "6"))
        b = F.LagrangeBasis("GLL", p + 1)
        disc = F.MultielementDisc(mesh, F.StdHex(b, F.DGSEMrec(b), eq.nvariables), eq,
                                  F.SplitDivOperator(F.ChandrasekharAverage(), F.LxF(F.ChandrasekharAverage(), 1.0)),
                                  {})
        # the vortex plus a 1e-3 smooth perturbation of every primitive variable: the plain vortex
        # is symmetric, its interface wave speeds tie exactly where LxF's max has a kink
        P = eq.vars_cons2prim(F.initial.taylor_green(eq, disc.coords, mach=mach))
        X = disc.coords
        for v in range(5):
            k = prng.integers(1, 3, size=3)
            ph = prng.uniform(0, 2 * math.pi, size=3)
            wave = np.prod([np.sin(k[i] * X[:, i] + ph[i]) for i in range(3)], axis=0)
            P[:, v] += 1e-3 * (np.max(np.abs(P[:, v])) if v in (0, 4) else 1.0) * wave
        Q0 = np.asfortranarray(eq.vars_prim2cons(P))
        rho_t = Q0[:, 0] * (1.0 + 0.01 * np.sin(X[:, 0] + rng.uniform(0, 6)) * np.sin(X[:, 1]) * np.cos(X[:, 2]))
        out.append(dict(disc=disc, Q0=Q0, rho_t=rho_t, m=m, p=p, mach=mach))
    return out


def bench_adjoint_batch(nsteps=200, budget=120e9, count=64, nstreams=8, fd_instances=2, seed=505):
    """Forward and lockstep adjoint of the batched-adjoint configuration (200 SSP-RK3 steps at
    CFL 0.15 per instance, J_k = 1/2 Σ w (ρ(T) - ρt)², gradients with respect to U0 and c under a
    120 GB device-memory budget for snapshots and step scratch).  The forward is the same
    instances advanced by their own step graphs, each context on its own stream, all in flight
    together.  Central differences (h = 1e-6) check the gradients of the smallest instances."""
    import torch
    import flou_cuda as F
    torch.cuda.empty_cache()
    t_setup = time.perf_counter()
    insts = make_adjoint_batch(count, seed)
    setup_s = time.perf_counter() - t_setup
    discs = [x["disc"] for x in insts]
    for d in discs:
        d.ctx.set_dissipation(np.ones(d.mesh.nelements))
    Q0s = [torch.from_numpy(np.ascontiguousarray(x["Q0"].T)).cuda() for x in insts]
    dts = [0.15 * d.ctx.max_dt(q, 1.0) for d, q in zip(discs, Q0s)]   # p = 5 at Mach 0.05 needs <= 0.15
    rts = [torch.from_numpy(np.ascontiguousarray(x["rho_t"])).cuda() for x in insts]
    ws = [torch.from_numpy(np.tile(d.std.omega, d.mesh.nelements) * d.J).cuda() for d in discs]
    ndofs = sum(d.ndofs for d in discs)
    state_bytes = sum(d.ndofs * 5 * 8 for d in discs)
    work = [q.clone() for q in Q0s]

    def forward_all():
        for d, q, dt in zip(discs, work, dts):
            d.ctx.step_async(q, dt, nsteps)
        for d in discs:
            d.ctx.wait()

    for d, q, dt in zip(discs, work, dts):   # warm-up: graph capture of every instance
        d.ctx.step(q, dt, 1)
    for w_, q in zip(work, Q0s):
        w_.copy_(q)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    forward_all()
    torch.cuda.synchronize()
    fwd_s = time.perf_counter() - t0
    grads = [torch.empty_like(q) for q in Q0s]
    cgrads = [torch.empty(d.mesh.nelements, dtype=torch.float64, device="cuda") for d in discs]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    J, nfwd, nsnap = F.adjoint_solve_batch(discs, Q0s, dts, nsteps, int(budget), rts, ws, grads, cgrads,
                                           nstreams=nstreams)
    torch.cuda.synchronize()
    adj_s = time.perf_counter() - t0
    # J of the forward pass agrees with the adjoint's own forward
    jf = [float(0.5 * torch.sum(w_ * (q[0] - r) ** 2)) for w_, q, r in zip(ws, work, rts)]
    j_rel = max(abs(a - b) / abs(b) for a, b in zip(J, jf))
    rng = np.random.default_rng(seed + 1)
    errs = []
    order = sorted(range(count), key=lambda k: discs[k].ndofs)[:fd_instances]
    h = 1e-6
    for k in order:
        d, dt = discs[k], dts[k]

        def Jof(Q, cc):
            d.ctx.set_dissipation(cc)
            q = Q.clone()
            d.ctx.step(q, dt, nsteps)
            return float(0.5 * torch.sum(ws[k] * (q[0] - rts[k]) ** 2))

        c1 = np.ones(d.mesh.nelements)
        for _ in range(2):
            dQ = torch.from_numpy(rng.standard_normal(tuple(Q0s[k].shape))).cuda()
            dc = 0.1 * rng.standard_normal(c1.shape)
            fd = (Jof(Q0s[k] + h * dQ, c1 + h * dc) - Jof(Q0s[k] - h * dQ, c1 - h * dc)) / (2 * h)
            ours = float(torch.sum(grads[k] * dQ)) + float(np.sum(cgrads[k].cpu().numpy() * dc))
            errs.append(abs(ours - fd) / abs(fd))
        d.ctx.set_dissipation(c1)
    units = ndofs * 3 * nsteps
    return {"forward_s": fwd_s, "adjoint_s": adj_s, "ratio": adj_s / fwd_s, "instances": count, "ndofs": ndofs,
            "state_bytes": state_bytes, "budget_bytes": int(budget), "snapshots": nsnap,
            "recomputed_forward_steps": nfwd, "steps": nsteps, "streams": nstreams,
            "forward_value": units / fwd_s, "unit": UNIT, "J_rel_diff_vs_forward": j_rel,
            "fd_instances": [int(discs[k].ndofs) for k in order], "fd_max_rel_err": max(errs) if errs else None,
            "setup_s": setup_s,
            "orders": [x["p"] for x in insts], "m": [x["m"] for x in insts],
            "workload": "%d x 3D Euler TGV (+1e-3 perturbation) periodic m^3 hex, m~U{8..24}, p~U{3..5}, Mach~U(0.05,0.3), split "
                        "Chandrashekar + LxF(Chandrashekar), %d SSP-RK3 steps forward + adjoint, %.0f GB budget"
                        % (count, nsteps, budget / 1e9)}


def run_profile(which):
    """Two SSP-RK3 steps of one mesh on the device (the case the ncu captures use)."""
    import torch
    if which == "C":
        import flou_cuda as F
        insts = make_batched(256)
        Qs = [torch.from_numpy(np.ascontiguousarray(Q.T)).cuda() for _, Q in insts]
        dts = [0.2 * d.ctx.max_dt(q, 1.0) for (d, _), q in zip(insts, Qs)]
        batch = F.Batch([d for d, _ in insts], Qs, dts)
        batch.step(2)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "batched 256 x 2D Euler", "ndofs": sum(d.ndofs for d, _ in insts),
                          "steps": 2}))
        return 0
    if which in ("D", "E"):
        import flou_cuda as F
        if which == "D":   # the adjoint configuration's discretization, 20 steps, 4 snapshots
            eq = F.EulerEquation(2, 1.4)
            mesh = F.CartesianMesh((-5.0, -5.0), (5.0, 5.0), (64, 64))
            F.apply_periodicBCs(mesh, ("1", "2"), ("3", "4"))
            b = F.LagrangeBasis("GLL", 5)
            disc = F.MultielementDisc(mesh, F.StdQuad(b, F.DGSEMrec(b), 4), eq,
                                      F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)))
            Q0 = F.initial.isentropic_vortex(eq, disc.coords, (0.2, -0.3), beta=5.0, period=(10.0, 10.0))
            nsteps, nsnap, cfl = 20, 4, 0.4
        else:              # one batched-adjoint instance: 16^3 elements, p = 4, 10 steps, 3 snapshots
            x = make_adjoint_batch(1, seed=7, mmin=16, mmax=16)[0]
            disc, Q0 = x["disc"], x["Q0"]
            nsteps, nsnap, cfl = 10, 3, 0.15
        disc.ctx.set_dissipation(np.ones(disc.mesh.nelements))
        Qd = torch.from_numpy(np.ascontiguousarray(np.asarray(Q0).T)).cuda()
        dt = cfl * disc.ctx.max_dt(Qd, 1.0)
        rho_t = Qd[0].clone()
        w = torch.from_numpy(np.tile(disc.std.omega, disc.mesh.nelements) * disc.J).cuda()
        g = torch.empty_like(Qd)
        gc = torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
        J, nf = disc.ctx.adjoint_solve(Qd, dt, nsteps, nsnap, rho_t, w, g, gc)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "adjoint " + which, "ndofs": disc.ndofs, "steps": nsteps,
                          "recomputed": nf, "J": J}))
        return 0
    if which == "G":   # FP64 throughput probes: CUDA-core DFMA and tensor-core DMMA
        import ctypes
        import flou_cuda as F
        lib = F.load()
        g1, g2 = ctypes.c_double(), ctypes.c_double()
        st1 = lib.flou_fp64_peak(ctypes.byref(g1))
        st2 = lib.flou_fp64_dmma_peak(ctypes.byref(g2))
        print(json.dumps({"profile_case": "fp64 probes", "dfma_gflops": g1.value if st1 == 0 else None,
                          "dmma_gflops": g2.value if st2 == 0 else None}))
        return 0
    if which == "F":   # mesh A with the Zhang-Shu stage limiter (minval 1e-10), two steps
        disc, Q0 = make_tgv(32, 4)
        import flou_cuda as F
        Qd = torch.from_numpy(np.ascontiguousarray(Q0.T)).cuda()
        dt = 0.2 * disc.ctx.max_dt(Qd, 1.0)
        disc.ctx.set_limiter(F._lib.LIMITER_ZHANG_SHU, 1e-10)
        disc.ctx.step(Qd, dt, 2)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "tgv3d 32^3 p=3 + limiter", "ndofs": disc.ndofs, "steps": 2}))
        return 0
    if which == "J":   # the hybrid operator's adjoint on Gauss nodes: 12^3 p=5 TGV, 3 steps, every state kept
        import flou_cuda as F
        eq = F.EulerEquation(3, 1.4)
        mesh = F.CartesianMesh((0.0,) * 3, (2 * math.pi,) * 3, (12,) * 3)
        F.apply_periodicBCs(mesh, ("1", "2"), ("3", "4"), ("5", "6"))
        b = F.LagrangeBasis("GL", 6)
        op = F.HybridDivOperator(F.MatrixDissipation(F.ChandrasekharAverage(), 1.0), 1.0)
        disc = F.MultielementDisc(mesh, F.StdHex(b, F.DGSEMrec(b), 5), eq, op, {})
        Qd = torch.from_numpy(np.ascontiguousarray(F.initial.taylor_green(eq, disc.coords, mach=0.1).T)).cuda()
        dt = TGV_CFL * disc.ctx.max_dt(Qd, 1.0)
        rho_t = (Qd[0] * 1.01).contiguous()
        w = torch.from_numpy(np.tile(disc.std.omega, disc.mesh.nelements) * disc.J).cuda()
        g = torch.empty_like(Qd)
        J, nf = disc.ctx.adjoint_solve(Qd, dt, 3, 2, rho_t, w, g)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "adjoint J: hybrid MatrixDissipation on Gauss nodes", "ndofs": disc.ndofs,
                          "steps": 3, "recomputed": nf, "J": J}))
        return 0
    if which in ("H", "I"):   # mesh B, MatrixDissipation (Shockwave2D's flux): H the hybrid operator on
        import flou_cuda as F    # Gauss-Lobatto nodes, I the split form on Gauss nodes
        eq = F.EulerEquation(3, 1.4)
        mesh = F.CartesianMesh((0.0,) * 3, (2 * math.pi,) * 3, (16,) * 3)
        F.apply_periodicBCs(mesh, ("1", "2"), ("3", "4"), ("5", "6"))
        b = F.LagrangeBasis("GLL" if which == "H" else "GL", 8)
        md = F.MatrixDissipation(F.ChandrasekharAverage(), 1.0)
        op = F.HybridDivOperator(md, 1.0) if which == "H" else F.SplitDivOperator(md)
        disc = F.MultielementDisc(mesh, F.StdHex(b, F.DGSEMrec(b), 5), eq, op, {})
        Qd = torch.from_numpy(np.ascontiguousarray(F.initial.taylor_green(eq, disc.coords, mach=0.1).T)).cuda()
        dt = 0.2 * disc.ctx.max_dt(Qd, 1.0)
        disc.ctx.step(Qd, dt, 2)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "tgv3d 16^3 p=7 %s MatrixDissipation" % ("hybrid GLL" if which == "H" else
                                                                                  "split GL"),
                          "ndofs": disc.ndofs, "steps": 2}))
        return 0
    nel, n = (32, 4) if which == "A" else (16, 8)
    disc, Q0 = make_tgv(nel, n)
    Qd = torch.from_numpy(np.ascontiguousarray(Q0.T)).cuda()
    dt = TGV_CFL * disc.ctx.max_dt(Qd, 1.0)
    disc.ctx.step(Qd, dt, 2)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": "tgv3d %d^3 p=%d" % (nel, n - 1), "ndofs": disc.ndofs, "steps": 2}))
    return 0


def bench_operators(nel=16, n=8):
    """Kernel cost of the operator variants on mesh B's size (16³ hexahedra, p = 7, TGV Mach 0.1):
    the split form and the hybrid (telescopic subcell) operator with MatrixDissipation, as the
    reference's Shockwave2D test uses them, on Gauss-Lobatto and on Gauss nodes.  CUDA-event
    times of single face and element launches (stage 2), and DOF·stage-updates/s of one stage."""
    import torch
    import flou_cuda as F
    eq = F.EulerEquation(3, 1.4)
    md = F.MatrixDissipation(F.ChandrasekharAverage(), 1.0)
    out = {}
    for basis in ("GLL", "GL"):
        for name, op in (("split", F.SplitDivOperator(md)), ("hybrid", F.HybridDivOperator(md, 1.0))):
            mesh = F.CartesianMesh((0.0,) * 3, (2 * math.pi,) * 3, (nel,) * 3)
            F.apply_periodicBCs(mesh, ("1", "2"), ("3", "4"), ("5", "6"))
            b = F.LagrangeBasis(basis, n)
            disc = F.MultielementDisc(mesh, F.StdHex(b, F.DGSEMrec(b), 5), eq, op, {})
            q = torch.from_numpy(np.ascontiguousarray(F.initial.taylor_green(eq, disc.coords, mach=0.1).T)).cuda()
            fms, ems = disc.ctx.time_kernels(q, nrep=3)
            out["%s_%s" % (name, basis)] = {"face_ms": fms, "elem_ms": ems,
                                            "value": disc.ndofs / ((fms + ems) * 1e-3), "unit": UNIT}
            del disc, q
    out["workload"] = "16^3 p=7 TGV M0.1, MatrixDissipation(Chandrashekar) interface (and subcell FV) flux"
    return out


def bench_adjoint_operators(nel=12, n=6, nsteps=10):
    """Adjoint/forward time of the operator variants the adjoint differentiates, on one 3D
    Taylor-Green mesh of nel³ hexahedra at p = n-1 (Mach 0.1, periodic; the general-geometry
    case: a perturbed box of rotated hexahedra with outflow boundaries): `nsteps` steps forward
    (flou_step) against the adjoint solve with every state kept (nsnap = nsteps - 1, so the
    ratio is the cost of the stage recomputation and the adjoint stages, not of the schedule)."""
    import torch
    import flou_cuda as F
    eq = F.EulerEquation(3, 1.4)
    md = F.MatrixDissipation(F.ChandrasekharAverage(), 1.0)
    cases = [
        ("split_hllc_GLL", "GLL", lambda: F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC()), False, None),
        ("split_hllc_GL", "GL", lambda: F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC()), False, None),
        ("strong_hllc_GL", "GL", lambda: F.StrongDivOperator(F.HLLC()), False, None),
        ("hybrid_md_GLL", "GLL", lambda: F.HybridDivOperator(md, 1.0), False, None),
        ("hybrid_md_GL", "GL", lambda: F.HybridDivOperator(md, 1.0), False, None),
        ("split_hllc_general", "GLL", lambda: F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC()), True, None),
        ("split_hllc_GLL_ORK256", "GLL", lambda: F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC()), False,
         F.ORK256()),
    ]
    out = {}
    for name, basis, op, general, lsrk in cases:
        b = F.LagrangeBasis(basis, n)
        std = F.StdHex(b, F.DGSEMrec(b), 5)
        if general:
            mesh = F.perturbed_box(3, nel, (0.0,) * 3, (2 * math.pi,) * 3, amp=0.1, seed=3)
            disc = F.MultielementDisc(mesh, std, eq, op(), {str(k): F.EulerOutflowBC() for k in range(1, 7)})
        else:
            mesh = F.CartesianMesh((0.0,) * 3, (2 * math.pi,) * 3, (nel,) * 3)
            F.apply_periodicBCs(mesh, ("1", "2"), ("3", "4"), ("5", "6"))
            disc = F.MultielementDisc(mesh, std, eq, op(), {})
        q0 = torch.from_numpy(np.ascontiguousarray(F.initial.taylor_green(eq, disc.coords, mach=0.1).T)).cuda()
        if lsrk is not None:
            disc.ctx.set_integrator(lsrk.A, lsrk.B)
        dt = TGV_CFL * disc.ctx.max_dt(q0, 1.0)
        rho_t = (q0[0] * 1.01).contiguous()
        w = torch.from_numpy(np.tile(disc.std.omega, disc.mesh.nelements) * disc.J).cuda()
        g = torch.empty_like(q0)

        def forward():
            q = q0.clone()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            disc.ctx.step(q, dt, nsteps)
            torch.cuda.synchronize()
            return (time.perf_counter() - t0) * 1e3

        def adjoint():
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            disc.ctx.adjoint_solve(q0, dt, nsteps, nsteps - 1, rho_t, w, g)
            torch.cuda.synchronize()
            return (time.perf_counter() - t0) * 1e3

        forward(), adjoint()   # warm-up (graph capture, allocations)
        fms = min(forward() for _ in range(3))
        ams = min(adjoint() for _ in range(3))
        out[name] = {"forward_ms": fms, "adjoint_ms": ams, "ratio": ams / fms, "ndofs": disc.ndofs}
        if lsrk is not None:
            disc.ctx.set_integrator(None)
        del disc, q0, g
    out["workload"] = ("3D TGV M0.1, %d^3 hexahedra at p=%d (general: perturbed rotated hexahedra, outflow), "
                       "split Chandrashekar + HLLC unless named, %d steps, every state kept" % (nel, n - 1, nsteps))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-curvilinear", action="store_true")
    ap.add_argument("--no-adjoint-batch", action="store_true",
                    help="skip the batched-adjoint configuration (64 3D instances, 200 steps, 120 GB budget; about "
                         "four minutes)")
    ap.add_argument("--adjoint-batch-only", action="store_true", help="run only the batched-adjoint configuration")
    ap.add_argument("--profile", choices=["A", "B", "C", "D", "E", "F", "G", "H", "I", "J"], default=None,
                    help="profiling case: two SSP-RK3 steps of mesh A (32^3 p=3), B (16^3 p=7) or the batched "
                         "configuration C (256 instances, one persistent launch per stage, default tiling); "
                         "adjoint solves D (2D 64^2 p=4, 20 steps) and E (3D split 16^3 p=4, 10 steps); F: mesh A with the "
                         "Zhang-Shu stage limiter; G: the FP64 DFMA and DMMA throughput probes; H: mesh B with the "
                         "hybrid operator and MatrixDissipation, I: the same on Gauss nodes with the split form; J: "
                         "the hybrid operator's adjoint on Gauss nodes (3D 12^3 p=5, 3 steps)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile:
        return run_profile(args.profile)

    import torch
    import flou_cuda as F

    if args.adjoint_batch_only:
        print(json.dumps({"adjoint_batch": bench_adjoint_batch()}))
        return 0

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    steps, warmup = args.steps, max(args.warmup, 3)
    meshes = []
    for nel, n in ((32, 4), (16, 8)):
        disc, Q0 = make_tgv(nel, n)
        ctx = disc.ctx
        Qd = torch.from_numpy(np.ascontiguousarray(Q0.T)).cuda()
        dt = TGV_CFL * ctx.max_dt(Qd, 1.0)
        meshes.append(dict(name="%dc_p%d" % (nel, n - 1), disc=disc, ctx=ctx, Q0=Q0, Qd=Qd, dt=dt, ndofs=disc.ndofs))
    stream = torch.cuda.current_stream()
    for m in meshes:
        m["ctx"].set_stream(stream.cuda_stream)
    ndofs = sum(m["ndofs"] for m in meshes)

    fp64_peak = dmma_peak = None
    try:
        import ctypes
        g = ctypes.c_double()
        if F.load().flou_fp64_peak(ctypes.byref(g)) == 0:
            fp64_peak = g.value
        if F.load().flou_fp64_dmma_peak(ctypes.byref(g)) == 0:
            dmma_peak = g.value
    except Exception:
        pass

    # ---- value: device-resident ----
    # The two meshes are independent: each runs on its own stream, pipelined per mesh through the
    # asynchronous call (a mesh's next step is queued once its previous one has returned and its
    # status has been checked), so one mesh's kernels fill the other's tail waves.  Device time
    # from an event on the main stream to one that waits for both mesh streams.
    mstreams = [torch.cuda.Stream() for _ in meshes]
    for m, st in zip(meshes, mstreams):
        m["ctx"].set_stream(st.cuda_stream)

    def pipelined(nsteps):
        for s in range(nsteps):
            for m, st in zip(meshes, mstreams):
                if s > 0:
                    m["ctx"].wait()
                with torch.cuda.stream(st):
                    m["ctx"].step_async(m["Qd"], m["dt"], 1)
        for m in meshes:
            m["ctx"].wait()

    pipelined(warmup)
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    time.sleep(0.3)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for st in mstreams:
        st.wait_event(e0)
    pipelined(steps)
    for st in mstreams:
        ev = torch.cuda.Event()
        ev.record(st)
        stream.wait_event(ev)
    e1.record(stream)
    barrier()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    value, ms = replica_throughput(ms, ndofs * 3 * steps, dist, "cuda")
    for m in meshes:
        m["ctx"].set_stream(stream.cuda_stream)

    # ---- per-kernel timing for the roofline (CUDA events around single launches) ----
    kern = {}
    for m in meshes:
        fms, ems = m["ctx"].time_kernels(m["Qd"], nrep=3)
        kern[m["name"]] = {"face_ms": fms, "elem_ms": ems, "ndofs": m["ndofs"]}
    tot = {k: 3 * (v["face_ms"] + v["elem_ms"]) for k, v in kern.items()}
    dom = max(kern, key=lambda k: kern[k]["elem_ms"])
    dk = kern[dom]
    algo_bytes = BYTES_PER_DOF_STAGE * dk["ndofs"]
    achieved = algo_bytes / (dk["elem_ms"] * 1e-3) / 1e9
    peaks = {}
    pp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pp):
        peaks = json.load(open(pp))
    hbm_peak = peaks.get("hbm_gbs")
    prof = load_profile_summary().get(dom, {})
    traffic = prof.get("dram_bytes_per_dof_stage")   # ncu, stage-2 launch of the same kernel
    fp64_ops = prof.get("fp64_flops_per_dof_stage")   # executed FP64 flops (2 per FMA), ncu
    # The element kernel is bound by the FP64 pipe (2 DFMA lanes per SM per cycle on GB300), not by
    # HBM: the roofline is the executed FP64 rate (ncu's executed FP64 flops per DOF of the same
    # kernel, 2 per DFMA, times the DOFs of one launch, over its CUDA-event launch time) against
    # the DFMA peak measured by the in-run probe (MEASURED_PEAKS.json carries no FP64 figure); the
    # HBM fraction of the compulsory state traffic is reported beside it.
    fp64_achieved = (fp64_ops * dk["ndofs"] / (dk["elem_ms"] * 1e-3) / 1e12) if fp64_ops else None
    fp64_peak_t = fp64_peak / 1e3 if fp64_peak else None
    roofline = {
        "kernel": "elem_split_kernel<3,%d,Euler,Chandrashekar> (%s)" % (int(dom[-1]) + 1, dom),
        "bound": "fp64", "achieved": fp64_achieved, "peak": fp64_peak_t, "unit": "TFLOP/s",
        "frac": (fp64_achieved / fp64_peak_t) if (fp64_achieved and fp64_peak_t) else None,
        "peak_source": "in-run FP64 DFMA throughput probe (flou_fp64_peak), measured this run",
        "flops_source": "profiles/tgv3d_split_elem_kernel.json: ncu executed FP64 flops (2 per DFMA) of the "
                        "stage-2 launch, per DOF, times the DOFs of one launch",
        "executed_fp64_flops_per_dof_stage": fp64_ops,
        "dmma_peak_tflops": dmma_peak / 1e3 if dmma_peak else None,
        "traffic": (traffic * dk["ndofs"]) if traffic else None,
        "traffic_source": "profiles/tgv3d_split_elem_kernel.json: ncu dram__bytes_read+write of the stage-2 launch",
        "hbm_achieved_gbs": achieved, "hbm_peak_gbs": hbm_peak,
        "hbm_frac": (achieved / hbm_peak) if hbm_peak else None,
        "hbm_peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if hbm_peak else None,
        "algorithmic_bytes_per_launch": algo_bytes,
        "launch_ms": dk["elem_ms"],
        "kernels": kern,
    }

    # ---- general geometry: the curvilinear kernels on mesh A's size ----
    curvilinear = None
    if not args.no_curvilinear:
        try:
            curvilinear = bench_curvilinear(steps, warmup, stream, kern[meshes[0]["name"]])
        except Exception as exc:   # reported, not fatal to the bench line
            curvilinear = {"error": str(exc)}

    operators = None
    if not args.no_curvilinear:
        try:
            operators = bench_operators()
        except Exception as exc:   # reported, not fatal to the bench line
            operators = {"error": str(exc)}
        if not args.no_adjoint:
            try:
                operators["adjoint"] = bench_adjoint_operators()
            except Exception as exc:   # reported, not fatal to the bench line
                operators["adjoint"] = {"error": str(exc)}

    # ---- cost of the Zhang-Shu stage limiter (minval 1e-10, as examples/src/3D_Euler.jl:76) ----
    limiter = None
    try:
        m0 = meshes[0]
        q = m0["Qd"].clone()
        res = {}
        for tag, on in (("off", False), ("on", True)):
            m0["ctx"].set_limiter(F._lib.LIMITER_ZHANG_SHU if on else F._lib.LIMITER_NONE, 1e-10)
            m0["ctx"].step(q, m0["dt"], 2)   # capture
            torch.cuda.synchronize()
            e0.record(stream)
            m0["ctx"].step(q, m0["dt"], steps)
            e1.record(stream)
            torch.cuda.synchronize()
            res[tag] = e0.elapsed_time(e1) / steps
        m0["ctx"].set_limiter(F._lib.LIMITER_NONE)
        limiter = {"mesh": m0["name"], "ms_per_step_off": res["off"], "ms_per_step_on": res["on"],
                   "overhead": res["on"] / res["off"] - 1.0, "minval": 1e-10}
    except Exception as exc:   # reported, not fatal to the bench line
        limiter = {"error": str(exc)}

    # ---- e2e: through the public API with pinned host buffers ----
    hosts = []
    for m in meshes:
        m["ctx"].set_stream(0)
        h = torch.from_numpy(np.ascontiguousarray(m["Q0"].T)).pin_memory()
        hosts.append(h)
        m["ctx"].step(h, m["dt"], 1)   # warm the host-pointer path
    barrier()
    t0 = time.perf_counter()
    for s in range(steps):
        # each mesh on its own stream, pipelined per mesh: a mesh's next step (copy in, stages,
        # copy out) is queued as soon as its previous one has returned, so its copies overlap
        # the other mesh's kernels
        for m, h in zip(meshes, hosts):
            if s > 0:
                m["ctx"].wait()
            m["ctx"].step_async(h, m["dt"], 1)
    for m in meshes:
        m["ctx"].wait()
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_value, _ = replica_throughput(e2e_s * 1e3, ndofs * 3 * steps, dist, "cuda")
    state_bytes = sum(m["ndofs"] * NV * 8 for m in meshes)
    e2e = {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": state_bytes, "d2h_bytes_per_step": state_bytes}

    batched = None
    if not args.no_batched:
        batched = bench_batched(steps, warmup)
        units = batched["ndofs"] * 3
        batched["value"], _ = replica_throughput(batched["ms_per_step"], units, dist, "cuda")
        batched["serial_value"], _ = replica_throughput(batched["serial_ms_per_step"], units, dist, "cuda")
        batched["speedup_vs_serial"] = batched["value"] / batched["serial_value"]

    adjoint = None
    if not args.no_adjoint:
        adjoint = bench_adjoint()

    adjoint_batch = None
    if not args.no_adjoint_batch and world == 1:
        for m in meshes:   # the batched adjoint's budget wants the device memory of the headline meshes back
            m["ctx"].set_stream(0)
        adjoint_batch = bench_adjoint_batch()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, sec, nd = cpu_oracle_rate(8, 1, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "8 SSP-RK3 steps of the workload's two meshes (32^3 p=3 and 16^3 p=7, %d nodes), each from "
                         "the initial state, %.1f s wall" % (nd, sec)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps, "warmup": warmup,
            "ms_per_step": ms / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": workload_config(world),
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "batched": batched, "adjoint": adjoint,
            "adjoint_batch": adjoint_batch, "limiter": limiter, "curvilinear": curvilinear, "operators": operators,
            "gpu_launches": steps * 6 * len(meshes), "clocks": clk,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
