#!/usr/bin/env python
"""MAC-projection benchmark on GB300: MAC solves/s at 256^3 to 1e-10 relative residual.

One step = one complete MAC projection (Source/macproject.f90:51-328: beta0 scaling, RHS,
face coefficients, multigrid to ||f - L phi|| <= 1e-10 ||f||, velocity correction) of the
3-D 256^3 stratified-atmosphere workload (8 boxes of 128^3, periodic x/y, slip walls in z,
rho0 = 1e7 exp(-z/H), H = 0.25, 1% lognormal density noise, |k| <= 16 velocity modes).
Inputs are seeded synthetic data (no public dataset exists for this path).

value  : mixed-precision solves/s (FP32 V-cycles inside FP64 iterative refinement), inputs
         resident in HBM, CUDA events on the library's stream around K steps.
fp64   : the plain FP64 solve timed the same way.
e2e    : the same metric through the public C ABI (mac_macproject) with host (pinned) per-box
         fabs: every step copies its inputs host->device and its result device->host.
roofline: the finest-level red/black half-sweeps of the mixed solve, timed live with
         CUDA events recorded inside the V-cycle graph over the timed region.
--impl reference: the CPU oracle (C++/OpenMP restatement of MAESTRO's FP64 solve; the Fortran
         reference cannot be built here) on the host cores.

Multi-GPU: the projection does not shard without a halo exchange; N ranks run N independent
replicas (weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MAC solves/s at 256^3 to 1e-10 rel resid: mixed vs FP64 GPU; % HBM peak"
UNIT = "solves/s"
CONFIG_KEY = "3d_256"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default=CONFIG_KEY)
    ap.add_argument("--workload", default="mac", choices=["mac", "amr", "hg"],
                    help="mac: the MAC projection headline (default); amr: the two-level "
                         "projection; hg: the nodal projection")
    ap.add_argument("--hg-n", type=int, default=256,
                    help="--workload hg: cells per direction (default 256, the bench workload; "
                         "smaller cubes for profiling captures)")
    ap.add_argument("--e2e-steps", type=int, default=24)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the other workload configurations (2-D 128^2, 512^3 mixed, "
                         "384^3 stiff, 256^3 adjoint)")
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--inner", type=int, default=None,
                    help="mixed precision: most FP32 V-cycles per FP64 refinement step")
    ap.add_argument("--fused-sweep", action="store_true",
                    help="mixed precision: one kernel per finest-level red/black sweep "
                         "(mac_opts.fused_sweep)")
    ap.add_argument("--fixed-inner", action="store_true",
                    help="mixed precision: always --inner V-cycles per step (no adaptive count)")
    return ap.parse_args()


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---- clocks sampled during the timed region ---------------------------------------------------
class _Nvml:
    """Read-only NVML queries through ctypes (SM clock, its maximum, clock event reasons)."""
    SM = 1
    BITS = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown",
            0x4: "sw_power_cap"}

    def __init__(self, torch_index):
        import ctypes
        self.c = ctypes
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        self.lib = lib
        self.h = ctypes.c_void_p()
        ok = False
        try:
            import torch
            uuid = getattr(torch.cuda.get_device_properties(torch_index), "uuid", None)
            if uuid is not None:
                ok = lib.nvmlDeviceGetHandleByUUID(("GPU-" + str(uuid)).encode(),
                                                   ctypes.byref(self.h)) == 0
        except Exception:
            ok = False
        if not ok and lib.nvmlDeviceGetHandleByIndex_v2(torch_index, ctypes.byref(self.h)) != 0:
            raise RuntimeError("no NVML handle")
        self.reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        v = ctypes.c_uint()
        self.max_sm = float(v.value) if lib.nvmlDeviceGetMaxClockInfo(
            self.h, self.SM, ctypes.byref(v)) == 0 else None

    def sample(self):
        c = self.c
        v, r = c.c_uint(), c.c_ulonglong()
        sm = float(v.value) if self.lib.nvmlDeviceGetClockInfo(self.h, self.SM, c.byref(v)) == 0 \
            else None
        bits = r.value if self.reasons_fn(self.h, c.byref(r)) == 0 else 0
        return sm, {nm for b, nm in self.BITS.items() if bits & b}


class Clocks:
    """SM clocks and clock event reasons sampled while the timed region runs: NVML polled from a
    thread (read-only queries; every 5 ms by default, every 100 ms around the end-to-end calls,
    whose host-side API calls a tighter poll was seen to delay), else nvidia-smi at its 200 ms
    period."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index, period_s=0.005):
        self.period = period_s
        self.proc = None
        self.path = None
        self.gpu = gpu_index
        self.nvml = None
        self.thread = None
        try:
            self.nvml = _Nvml(gpu_index)
        except Exception:
            self.nvml = None

    def start(self):
        if self.nvml is not None:
            import threading
            self.sm, self.reasons = [], set()
            self.halt = threading.Event()

            def run():
                while not self.halt.is_set():
                    sm, rs = self.nvml.sample()
                    if sm is not None:
                        self.sm.append(sm)
                    self.reasons |= rs
                    self.halt.wait(self.period)
            self.thread = threading.Thread(target=run, daemon=True)
            self.thread.start()
            return
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.thread is not None:
            self.halt.set()
            self.thread.join()
            sm = self.sm
            return {"sm_mhz": statistics.median(sm) if sm else None,
                    "sm_max_mhz": self.nvml.max_sm, "reasons": sorted(self.reasons),
                    "samples": len(sm), "source": "nvml"}
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for ln in f:
                p = [x.strip() for x in ln.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    smax.append(float(p[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, p[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "source": "nvidia-smi"}


# ---- the workload's config object, identical in both arms ------------------------------------
def link_rates(dev, nbytes=1 << 29, reps=3):
    """Host<->device copy rates of this machine (one page-locked buffer, one device buffer, the
    copy engines, current stream): what bounds the end-to-end call's input and output copies."""
    import torch
    n = nbytes // 8
    h = torch.empty(n, dtype=torch.float64, pin_memory=True)
    d = torch.empty(n, dtype=torch.float64, device=dev)
    out = {}
    for name, dst, src in (("h2d_gbs", d, h), ("d2h_gbs", h, d)):
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            dst.copy_(src, non_blocking=True)
        e1.record()
        e1.synchronize()
        out[name] = round(reps * nbytes / (e0.elapsed_time(e1) * 1e-3) / 1e9, 1)
    del h, d
    return out


def mac_config(name, n, box, world):
    # a timed step's own inputs: the face velocities and phi, a distinct copy per step
    cells = 1
    for v in n:
        cells *= v
    faces = sum(cells // v * (v + 1) for v in n)
    mb = 8 * (faces + cells) / 1e6
    size = f"{mb / 1e3:.2g} GB" if mb >= 100 else f"{mb:.3g} MB"
    where = "larger than" if mb > 129 else "within"
    return {"workload": name, "n": list(n), "box": list(box), "rel_eps": 1e-10,
            "l2": f"inputs {where} L2 ({size} per step, a distinct copy per step)",
            "parallelism": f"replicas x{world}"}


# ---- reference arm: the CPU oracle ------------------------------------------------------------
def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    import oracle as O
    from maestro_gb300.inputs import CONFIGS, make_case
    kw = dict(CONFIGS[args.config])
    # every step is one full solve of the benchmark configuration itself (256^3, 8 boxes of
    # 128^3): the same inputs, hierarchy and tolerance as the GPU arm
    c = make_case(name=args.config, seed=args.seed, **kw)
    nlev = O.nlevels_for_boxes([c.box])
    # every host core (a launcher may have set OMP_NUM_THREADS=1 for its ranks)
    threads = host_cores()

    def step():
        t = time.perf_counter()
        _, _, st = O.macproject(c.umac, c.phi0, c.rho, c.dx, c.bc_lo, c.bc_hi, macrhs=c.macrhs,
                                beta0=c.beta0, beta0_edge=c.beta0_edge, nlevels=nlev,
                                threads=threads)
        assert st["status"] == 0 and st["rel_resid"] <= 1e-10
        return time.perf_counter() - t

    for _ in range(args.warmup):
        step()
    ts = [step() for _ in range(args.steps)]
    secs = sum(ts)
    value = args.steps / secs
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded stratified atmosphere)",
        "config": mac_config(args.config, c.n, c.box, world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"per step one full {'x'.join(map(str, c.n))} solve of the "
                                   f"benchmark workload (the same configuration as the GPU arm); "
                                   f"C++/OpenMP FP64 restatement of MAESTRO's macproject + "
                                   f"FBoxLib MG (Fortran reference unbuildable)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))
    return 0



# ---- the other rows: multi-level and nodal projections (run with --workload) -------------------
AMR_N0, AMR_BOX, AMR_FINE = (128, 128, 128), (64, 64, 64), ((64, 64, 64), (191, 191, 191))


def _amr_inputs(n0, fine, seed):
    from maestro_gb300.inputs import make_amr_case
    return make_amr_case(name="amr_bench", dm=3, n0=n0, boxes=[[], [fine]], kmax=4, noise=0.05,
                         seed=seed)


def _hg_inputs(n, seed):
    import numpy as np
    rng = np.random.default_rng(seed)
    z = (np.arange(n[-1]) + 0.5) / n[-1]
    rho0 = 1e7 * np.exp(-z / 0.25)
    rho = rho0.reshape(1, 1, -1) * np.exp(0.01 * rng.standard_normal(n))
    u = 1e6 * rng.standard_normal(tuple(n) + (3,))
    gpi = np.zeros(tuple(n) + (3,))
    b0 = np.broadcast_to((rho0 ** (1 / 1.4)).reshape(1, 1, -1), n).copy()
    pi = np.zeros(tuple(v + 1 for v in n))
    return dict(unew=u, gpi=gpi, rhohalf=rho, beta0=b0, pi=pi)


def run_extra(args, rank, world, local):
    """One JSON line for the multi-level (amr) or nodal (hg) projection."""
    hg_n = (args.hg_n,) * 3
    hg_box = tuple(max(v // 2, 1) for v in hg_n)
    import numpy as np
    import oracle as O
    if args.workload == "amr":
        metric = "two-level MAC solves/s (128^3 base + 128^3 patch at 2x) to MAESTRO's tolerance"
        cfg = {"workload": "amr_2lev", "n0": list(AMR_N0), "box": list(AMR_BOX),
               "fine_box": [list(AMR_FINE[0]), list(AMR_FINE[1])], "rel_eps": O.ml_rel_eps(2)}
        sample_n0, sample_fine = (32, 32, 32), ((16, 16, 16), (47, 47, 47))
        full_cells = np.prod(AMR_N0) + np.prod([b - a + 1 for a, b in zip(*AMR_FINE)])
        sample_cells = np.prod(sample_n0) + np.prod([b - a + 1 for a, b in zip(*sample_fine)])
    else:
        metric = (f"nodal (HG) projections/s at {args.hg_n}^3 (dense stencil, regular time step) "
                  "to 1e-12")
        cfg = {"workload": f"hg_{args.hg_n}", "n": list(hg_n), "box": list(hg_box), "rel_eps": O.EPS_HG,
               "stencil": "dense"}
        full_cells = np.prod(hg_n)
        sample_n = (64, 64, 64)
        sample_cells = np.prod(sample_n)
    threads = host_cores()
    sample_in = (_amr_inputs(sample_n0, sample_fine, args.seed) if args.workload == "amr"
                 else _hg_inputs(sample_n, args.seed))

    def cpu_step():
        t = time.perf_counter()
        if args.workload == "amr":
            c = sample_in
            st = O.macproject_ml(c.umac, c.phi0, c.rho, c.dx0, c.bc_lo, c.bc_hi, c.boxes,
                                 macrhs=c.macrhs, beta0=c.beta0, beta0_edge=c.beta0_edge,
                                 threads=threads)[2]
        else:
            h = sample_in
            bc = (O.BC_PER, O.BC_PER, O.BC_NEU)
            st = O.hgproject(h["unew"], h["unew"], h["gpi"], h["rhohalf"], h["pi"],
                             tuple(1.0 / v for v in sample_n), bc, bc, proj_type=O.HG_REGULAR,
                             dt=1e-3, beta0_cart=h["beta0"], threads=threads)[4]
        assert st["status"] == 0
        return time.perf_counter() - t

    sample = (f"per step one solve of the same workload at {sample_cells / full_cells:.4g} of the "
              f"cells, scaled by the cell ratio; the C++/OpenMP oracle (FBoxLib unbuildable)")
    if args.impl == "reference":
        if rank != 0:
            return 0
        for _ in range(args.warmup):
            cpu_step()
        secs = sum(cpu_step() for _ in range(args.steps))
        value = args.steps / secs * (sample_cells / full_cells)
        print(json.dumps({
            "impl": "reference", "metric": metric, "value": value, "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "config": cfg,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}))
        return 0

    import torch
    from maestro_gb300.build import build
    from maestro_gb300.macproject import BcTower, Layout, MacProjector
    build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    to_dev = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).transpose())).to(dev)  # noqa: E731
    nsteps = args.steps + args.warmup
    stats = []
    if args.workload == "amr":
        c = _amr_inputs(AMR_N0, AMR_FINE, args.seed + rank)
        lay = Layout.tiled(c.n0, AMR_BOX)
        # mixed precision: FP32 multi-level cycles under FP64 refinement (FP64 printed too)
        P = MacProjector(lay, c.dx0, BcTower(c.bc_lo, c.bc_hi), precision="mixed",
                         stream=stream.cuda_stream)
        P.set_amr(c.boxes)
        u0 = [[to_dev(x) for x in c.umac[l]] for l in range(2)]
        rho = [to_dev(r) for r in c.rho]
        rhs = [to_dev(m) for m in c.macrhs]
        b0 = [torch.from_numpy(b).to(dev) for b in c.beta0]
        b0e = [torch.from_numpy(b).to(dev) for b in c.beta0_edge]
        work = [([[x.clone() for x in u0[l]] for l in range(2)],
                 [torch.zeros_like(r) for r in rho]) for _ in range(nsteps)]

        def one(k):
            u, phi = work[k]
            return P.macproject_ml_dense([[x.data_ptr() for x in u[l]] for l in range(2)],
                                         [p.data_ptr() for p in phi], [r.data_ptr() for r in rho],
                                         macrhs=[m.data_ptr() for m in rhs],
                                         beta0=[b.data_ptr() for b in b0],
                                         beta0_edge=[b.data_ptr() for b in b0e], strict=True)
    else:
        h = _hg_inputs(hg_n, args.seed + rank)
        lay = Layout.tiled(hg_n, hg_box)
        # mixed precision: FP32 V-cycles under FP64 refinement (the FP64 rate is printed too)
        P = MacProjector(lay, tuple(1.0 / v for v in hg_n),
                         BcTower((-1, -1, 2), (-1, -1, 2)), precision="mixed",
                         stream=stream.cuda_stream)
        fields = {k: to_dev(v) for k, v in h.items()}
        work = [(fields["unew"].clone(), fields["gpi"].clone(), fields["pi"].clone())
                for _ in range(nsteps)]

        def one(k):
            u, g, pi = work[k]
            return P.hgproject_dense(4, 1e-3, u.data_ptr(), u.data_ptr(), g.data_ptr(),
                                     fields["rhohalf"].data_ptr(), pi.data_ptr(),
                                     beta0_cart=fields["beta0"].data_ptr(), rel_eps=O.EPS_HG,
                                     strict=True)
    for k in range(args.warmup):
        one(k)
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(args.warmup, nsteps):
        stats.append(one(k))
    e1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    ms = e0.elapsed_time(e1)
    roof, by_class = None, None
    if args.workload == "amr":
        # the dominant kernel's live launch time, after the timed region: one more projection
        # with CUDA events around the fine level's sweeps, on a fresh copy of the inputs
        P.set_opts(timing=1)
        u = [[x.clone() for x in u0[l]] for l in range(2)]
        phi = [torch.zeros_like(r) for r in rho]
        st = P.macproject_ml_dense([[x.data_ptr() for x in u[l]] for l in range(2)],
                                   [p.data_ptr() for p in phi], [r.data_ptr() for r in rho],
                                   macrhs=[m.data_ptr() for m in rhs],
                                   beta0=[b.data_ptr() for b in b0],
                                   beta0_edge=[b.data_ptr() for b in b0e], strict=True)
        P.set_opts(timing=0)
        torch.cuda.synchronize()
        del u, phi
        nl = st["ktime_launches"][0]
        by_class = {"fine_gs_ms": st["ktime_ms"][0], "fine_gs_launches": nl,
                    "solve_ms": st["solve_ms"]}
        if nl > 0:
            # the fine level's array box: its boxes' bounding box grown by one cell, clipped
            cells = 1
            for d in range(3):
                lo = max(AMR_FINE[0][d] - 1, 0)
                hi = min(AMR_FINE[1][d] + 1, 2 * AMR_N0[d] - 1)
                cells *= hi - lo + 1
            # one colour launch, per cell of the box (FP32): every cell's u (neighbours) 4 B, the
            # own colour's f and new u 2 + 2 B, the face coefficients 3 x 4 B, the mask 1 B
            alg = 21.0 * cells
            avg_ms = st["ktime_ms"][0] / nl
            achieved = alg / (avg_ms * 1e-3) / 1e9
            hbm_peak, peak_kind = peaks()
            roof = {"bound": "hbm", "kernel": "k_gsrb<float> (fine level, one colour of a red/black "
                    "sweep of the composite operator, FP32, natural layout, masked)",
                    "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                    "frac": achieved / hbm_peak, "traffic": None, "alg_bytes_per_launch": alg,
                    "avg_launch_ms": avg_ms, "launches": nl, "peak_kind": peak_kind}
    if args.workload == "hg":
        # the dominant kernel's live launch time, after the timed region: one more projection
        # with CUDA events around the finest level's sweeps and the FP64 defects (launched
        # uncaptured), on a fresh copy of the inputs
        P.set_opts(timing=1)
        u, g, pi = fields["unew"].clone(), fields["gpi"].clone(), fields["pi"].clone()
        st = P.hgproject_dense(4, 1e-3, u.data_ptr(), u.data_ptr(), g.data_ptr(),
                               fields["rhohalf"].data_ptr(), pi.data_ptr(),
                               beta0_cart=fields["beta0"].data_ptr(), rel_eps=O.EPS_HG,
                               strict=True)
        P.set_opts(timing=0)
        torch.cuda.synchronize()
        del u, g, pi
        by_class = {"finest_gs_ms": st["ktime_ms"][0], "finest_gs_launches": st["ktime_launches"][0],
                    "fp64_defect_ms": st["ktime_ms"][5], "fp64_defects": st["ktime_launches"][5],
                    "solve_ms": st["solve_ms"]}
        nl = st["ktime_launches"][0]
        if nl > 0:
            nodes = 1
            for v in hg_n:
                nodes *= v + 1
            # one launch = one slab parity of a sweep, per level node in FP32: the own slabs'
            # phi, f and new phi (2 + 2 + 2 B), the other slabs' phi once (2 B), every cell's
            # sigma once (4 B): 12 B
            alg = 12.0 * nodes
            avg_ms = st["ktime_ms"][0] / nl
            achieved = alg / (avg_ms * 1e-3) / 1e9
            hbm_peak, peak_kind = peaks()
            roof = {"bound": "hbm", "kernel": "k_hg_gs_tile<float> (finest level, one slab-parity "
                    "launch of a Gauss-Seidel sweep: 4 colours in shared memory, FP32)",
                    "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                    "frac": achieved / hbm_peak, "traffic": None, "alg_bytes_per_launch": alg,
                    "avg_launch_ms": avg_ms, "launches": nl, "peak_kind": peak_kind}
            tp = os.path.join(ROOT, "profiles", "traffic.json")
            if os.path.exists(tp):
                with open(tp) as f:
                    tr = json.load(f).get("hg_gs_tile_fine")
                if tr:
                    roof["traffic"] = tr["dram_bytes_per_launch"] * nodes / tr["nodes"]
    P.close()
    K = args.steps
    value = world * K / (ms / 1e3)
    fp64 = None
    # the FP64 rate of the same workload (one untimed solve, then at least one timed)
    n64 = max(nsteps, 2)
    if args.workload == "hg":
        P = MacProjector(lay, tuple(1.0 / v for v in hg_n),
                         BcTower((-1, -1, 2), (-1, -1, 2)), precision="fp64",
                         stream=stream.cuda_stream)
        work = [(fields["unew"].clone(), fields["gpi"].clone(), fields["pi"].clone())
                for _ in range(n64)]
    else:
        P = MacProjector(lay, c.dx0, BcTower(c.bc_lo, c.bc_hi), precision="fp64",
                         stream=stream.cuda_stream)
        P.set_amr(c.boxes)
        work = [([[x.clone() for x in u0[l]] for l in range(2)],
                 [torch.zeros_like(r) for r in rho]) for _ in range(n64)]
    one(0)
    torch.cuda.synchronize()
    e0.record(stream)
    st64 = [one(k) for k in range(1, n64)]
    e1.record(stream)
    torch.cuda.synchronize()
    ms64 = e0.elapsed_time(e1) / (n64 - 1)
    P.close()
    fp64 = {"value": 1e3 / ms64, "unit": UNIT, "ms_per_step": ms64,
            "vcycles": st64[-1]["vcycles"], "rel_resid": st64[-1]["rel_resid"]}
    cpu = None
    if not args.no_cpu and rank == 0 and world == 1:
        secs = cpu_step()
        cpu = {"value": (sample_cells / full_cells) / secs, "unit": UNIT, "cores": threads,
               "kind": "port", "sample": sample}
    out = {"metric": metric, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
           "warmup": args.warmup, "ms_per_step": ms / K, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
           "config": cfg, "roofline": roof, "cpu_baseline": cpu, "e2e": None,
           "gpu_launches": sum(s["launches"] for s in stats),
           "vcycles": stats[-1]["vcycles"], "rel_resid": max(s["rel_resid"] for s in stats),
           "clocks": ck}
    out["fp64"] = fp64
    if by_class:
        out["ms_by_class"] = by_class
    out["dtype"] = "f32 V-cycles + f64 refinement"
    if rank == 0:
        print(json.dumps(out))
    return 0


# ---- the other workload configurations (2-D 128^2, 512^3 mixed, 384^3 stiff, 256^3 adjoint) ----
def measure_configs(dev, with_cpu=False, steps=3, warmup=1, seed=17):
    """Solves/s of every workload configuration on this GPU (device-resident inputs, CUDA events
    on the library's stream, a distinct input copy per timed solve), FP64 and mixed precision,
    with refinement / V-cycle counts and the mixed results' error against the FP64 GPU solve; the
    adjoint (forward + adjoint solve) of the 256^3 adjoint and 384^3 stiff configurations, FP64
    and FP32-smoothed (mixed context).  with_cpu: the 2-D configuration's CPU baseline (the
    oracle's own rate on the host cores).  Errors against the oracle are the GPU tests' business
    (tests/test_gpu_full_configs.py)."""
    import numpy as np
    import torch

    from maestro_gb300.inputs import cell_to_edge, config_case  # noqa: F401
    from maestro_gb300.macproject import BcTower, Layout, MacProjector

    stream = torch.cuda.current_stream(dev)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).transpose())).to(dev)  # noqa: E731

    def rel(a, b, demean=False):
        if demean:
            a, b = a - a.mean(), b - b.mean()
        return float((a - b).abs().max() / b.abs().max())

    def solves(c, precision, n_steps, rel_eps=1e-10):
        u0 = [t(a) for a in c.umac]
        rho, rhs = t(c.rho), t(c.macrhs)
        b0 = torch.from_numpy(c.beta0).to(dev)
        b0e = torch.from_numpy(c.beta0_edge).to(dev)
        work = [([x.clone() for x in u0], torch.zeros_like(rho)) for _ in range(n_steps)]
        P = MacProjector(Layout.tiled(c.n, c.box), c.dx, BcTower(c.bc_lo, c.bc_hi),
                         precision=precision, rel_eps=rel_eps, stream=stream.cuda_stream)
        sts = []
        try:
            def one(k):
                u, phi = work[k]
                return P.macproject_dense(u[0].data_ptr(), u[1].data_ptr(),
                                          u[2].data_ptr() if c.dm == 3 else 0, phi.data_ptr(),
                                          rho.data_ptr(), rhs.data_ptr(), b0.data_ptr(),
                                          b0e.data_ptr(), strict=True)
            for k in range(warmup):
                one(k)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for k in range(warmup, n_steps):
                sts.append(one(k))
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / (n_steps - warmup)
        finally:
            P.close()
        u, phi = work[-1]
        del work[:-1]
        return 1e3 / ms, sts[-1], u, phi

    def adjoints(c, precision, n_steps, rel_eps=1e-10):
        u = [t(a) for a in c.umac]
        w = [t(a) for a in c.w]
        du = [torch.zeros_like(x) for x in u]
        rho, rhs = t(c.rho), t(c.macrhs)
        b0 = torch.from_numpy(c.beta0).to(dev)
        b0e = torch.from_numpy(c.beta0_edge).to(dev)
        drinv, dmac = torch.zeros_like(rho), torch.zeros_like(rho)
        db0 = torch.zeros_like(b0)
        P = MacProjector(Layout.tiled(c.n, c.box), c.dx, BcTower(c.bc_lo, c.bc_hi),
                         precision=precision, rel_eps=rel_eps, stream=stream.cuda_stream)
        try:
            def one():
                return P.adjoint_dense([x.data_ptr() for x in u], rho.data_ptr(), rhs.data_ptr(),
                                       b0.data_ptr(), b0e.data_ptr(), [x.data_ptr() for x in w],
                                       [x.data_ptr() for x in du], drinv.data_ptr(),
                                       db0.data_ptr(), dmac.data_ptr(), 0)
            for _ in range(warmup):
                one()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(n_steps - warmup):
                st = one()
            torch.cuda.synchronize()
            secs = (time.perf_counter() - t0) / (n_steps - warmup)
        finally:
            P.close()
        return 1.0 / secs, st, du, dmac

    out = {}
    n_steps = warmup + steps

    # 2-D 128^2 FP64 (and mixed) against the oracle's own rate on the host cores
    c = config_case("2d_128", seed=seed)
    r64, st64, u64, p64 = solves(c, "fp64", n_steps)
    r32, st32, u32, p32 = solves(c, "mixed", n_steps)
    e2d = {"fp64": r64, "mixed": r32, "fp64_vcycles": st64["vcycles"],
           "mixed_vcycles": st32["vcycles"], "refine_iters": st32["refine_iters"],
           "u_err_mixed_vs_fp64": max(rel(a, b) for a, b in zip(u32, u64))}
    if with_cpu:
        import oracle as O
        nlev = O.nlevels_for_boxes([c.box])
        threads = host_cores()
        t0 = time.perf_counter()
        for _ in range(20):
            O.macproject(c.umac, c.phi0, c.rho, c.dx, c.bc_lo, c.bc_hi, macrhs=c.macrhs,
                         beta0=c.beta0, beta0_edge=c.beta0_edge, nlevels=nlev, threads=threads)
        e2d["cpu_baseline"] = {"value": 20 / (time.perf_counter() - t0), "unit": UNIT,
                               "cores": threads, "kind": "port",
                               "sample": "20 full 128^2 FP64 solves by the C++/OpenMP oracle"}
    out["2d_128"] = e2d
    del c

    # 512^3 mixed (and FP64)
    c = config_case("3d_512_mixed", seed=seed)
    r32, st32, u32, p32 = solves(c, "mixed", n_steps)
    r64, st64, u64, p64 = solves(c, "fp64", n_steps)
    e5 = {"mixed": r32, "fp64": r64, "mixed_over_fp64": r32 / r64,
          "refine_iters": st32["refine_iters"], "mixed_vcycles": st32["vcycles"],
          "fp64_vcycles": st64["vcycles"], "rel_resid_mixed": st32["rel_resid"],
          "phi_err_mixed_vs_fp64": rel(p32, p64, True),
          "u_err_mixed_vs_fp64": max(rel(a, b) for a, b in zip(u32, u64))}
    del u64, p64
    out["3d_512_mixed"] = e5
    del c, u32, p32
    torch.cuda.empty_cache()

    # 256^3 adjoint: forward + adjoint solve, FP64 and FP32-smoothed
    c = config_case("3d_256_adjoint", seed=seed)
    a64, sa64, du64, _ = adjoints(c, "fp64", n_steps)
    a32, sa32, du32, _ = adjoints(c, "mixed", n_steps)
    out["3d_256_adjoint"] = {
        "adjoints_per_s_fp64": a64, "adjoints_per_s_mixed": a32,
        "vcycles_fp64": sa64["vcycles"], "vcycles_mixed": sa32["vcycles"],
        "du_err_mixed_vs_fp64": max(rel(a, b) for a, b in zip(du32, du64)),
        "note": "one call = forward projection + adjoint solve + gradient kernels "
                "(host-timed around the call); FD checks in the GPU tests"}
    del c, du64, du32
    torch.cuda.empty_cache()

    # 384^3 stiff: mixed vs FP64 forward, then the FP32-smoothed adjoint
    c = config_case("3d_384_stiff", seed=seed)
    rng = np.random.default_rng(seed + 1000)
    c.w = [np.asfortranarray(rng.standard_normal(u.shape)) for u in c.umac]
    r32, st32, u32, p32 = solves(c, "mixed", n_steps)
    r64, st64, u64, p64 = solves(c, "fp64", n_steps)
    a32, sa32, du32, dm32 = adjoints(c, "mixed", n_steps)
    a64, sa64, du64, dm64 = adjoints(c, "fp64", n_steps)
    e6 = {"mixed": r32, "fp64": r64, "mixed_over_fp64": r32 / r64,
          "refine_iters": st32["refine_iters"], "mixed_vcycles": st32["vcycles"],
          "fp64_vcycles": st64["vcycles"], "rel_resid_mixed": st32["rel_resid"],
          "phi_err_mixed_vs_fp64": rel(p32, p64, True),
          "u_err_mixed_vs_fp64": max(rel(a, b) for a, b in zip(u32, u64)),
          "adjoints_per_s_mixed": a32, "adjoints_per_s_fp64": a64,
          "adjoint_mixed_over_fp64": a32 / a64,
          "adjoint_refine_iters_mixed": sa32["refine_iters"],
          "du_err_mixed_vs_fp64": max(rel(a, b) for a, b in zip(du32, du64)),
          "dmacrhs_err_mixed_vs_fp64": rel(dm32, dm64)}
    del u64, p64, du64, dm64
    out["3d_384_stiff"] = e6
    return out


# ---- our arm ----------------------------------------------------------------------------------
def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.workload != "mac":
        return run_extra(args, rank, world, local)
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import numpy as np
    import torch

    from maestro_gb300 import build as _build_mod  # noqa: F401
    from maestro_gb300 import capi
    from maestro_gb300.build import build
    from maestro_gb300.inputs import config_case
    from maestro_gb300.macproject import BcTower, Layout, MacProjector

    # inner-solve options: the library's defaults unless given
    inner_opts = {}
    if args.inner:
        inner_opts["inner_vcycles"] = args.inner
    if args.fixed_inner:
        inner_opts["adaptive_inner"] = 0
    if args.fused_sweep:
        inner_opts["fused_sweep"] = 1

    build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x):
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    c = config_case(args.config, seed=args.seed + rank)
    N = c.ncell
    stream = torch.cuda.current_stream(dev)
    to_dev = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).transpose())).to(dev)  # noqa: E731
    u0 = [to_dev(a) for a in c.umac]
    rho = to_dev(c.rho)
    rhs = to_dev(c.macrhs)
    b0 = torch.from_numpy(c.beta0).to(dev)
    b0e = torch.from_numpy(c.beta0_edge).to(dev)
    nsteps = args.steps + args.warmup
    work_u = [[torch.empty_like(x) for x in u0] for _ in range(nsteps)]
    work_phi = [torch.empty_like(rho) for _ in range(nsteps)]
    lay = Layout.tiled(c.n, c.box)
    bc = BcTower(c.bc_lo, c.bc_hi)

    def reset_inputs():
        for k in range(nsteps):
            for d in range(c.dm):
                work_u[k][d].copy_(u0[d])
            work_phi[k].zero_()
        torch.cuda.synchronize()

    def timed_run(precision, timing):
        P = MacProjector(lay, c.dx, bc, precision=precision, stream=stream.cuda_stream,
                         timing=int(timing), **inner_opts)
        reset_inputs()
        stats = []

        def one(k):
            u = work_u[k]
            st = P.macproject_dense(u[0].data_ptr(), u[1].data_ptr(),
                                    u[2].data_ptr() if c.dm == 3 else 0,
                                    work_phi[k].data_ptr(), rho.data_ptr(), rhs.data_ptr(),
                                    b0.data_ptr(), b0e.data_ptr(), strict=True)
            return st

        for k in range(args.warmup):
            one(k)
        barrier()
        clocks = Clocks(local)
        clocks.start()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(args.warmup, nsteps):
            stats.append(one(k))
        e1.record(stream)
        barrier()
        ck = clocks.stop()
        ms = e0.elapsed_time(e1)
        P.close()
        return max_over_ranks(ms), stats, ck

    ms_mixed, st_mixed, ck_mixed = timed_run("mixed", timing=True)
    ms_fp64, st_fp64, ck_fp64 = timed_run("fp64", timing=True)
    K = args.steps
    value = world * K / (ms_mixed / 1e3)
    fp64_value = world * K / (ms_fp64 / 1e3)

    # error of the mixed result against the FP64 GPU solve of the same inputs (last step)
    reset_inputs()
    Pm = MacProjector(lay, c.dx, bc, precision="mixed", stream=stream.cuda_stream,
                      **inner_opts)
    Pd = MacProjector(lay, c.dx, bc, precision="fp64", stream=stream.cuda_stream)
    ua, pa = work_u[0], work_phi[0]
    ub, pb = work_u[1], work_phi[1]
    Pm.macproject_dense(ua[0].data_ptr(), ua[1].data_ptr(), ua[2].data_ptr(), pa.data_ptr(),
                        rho.data_ptr(), rhs.data_ptr(), b0.data_ptr(), b0e.data_ptr())
    Pd.macproject_dense(ub[0].data_ptr(), ub[1].data_ptr(), ub[2].data_ptr(), pb.data_ptr(),
                        rho.data_ptr(), rhs.data_ptr(), b0.data_ptr(), b0e.data_ptr())
    torch.cuda.synchronize()
    da = pa - pa.mean()
    db = pb - pb.mean()
    phi_err = float((da - db).abs().max() / db.abs().max())
    u_err = max(float((x - y).abs().max() / y.abs().max()) for x, y in zip(ua, ub))
    Pm.close()
    Pd.close()

    # ---- roofline of the dominant kernel: the finest level's red/black sweeps (mixed, FP32) --
    hbm_peak, peak_kind = peaks()
    kt_ms = sum(s["ktime_ms"][capi.KT_NAMES.index("smooth")] for s in st_mixed)
    kt_n = sum(s["ktime_launches"][capi.KT_NAMES.index("smooth")] for s in st_mixed)
    nv = sum(s["vcycles"] for s in st_mixed)
    dopts = capi.default_opts(**inner_opts)
    omega = dopts.inner_omega
    sor = omega != 1.0
    sweeps_per_cycle = dopts.inner_nu1 + dopts.inner_nu2
    # the fused kernel runs one launch a sweep, the half-sweep kernels two
    fused = bool(dopts.fused_sweep) and kt_n == nv * sweeps_per_cycle
    if fused:
        # one whole sweep a launch, per cell of the level: e of both colours read (4 B; plain
        # Gauss-Seidel does not read the colour-0 old e: 2 B), rho (4 B) and f (4 B) read, e
        # written (4 B) = 16 B over-relaxed / 14 B Gauss-Seidel; the last pre-smoothing sweep of
        # each V-cycle also writes the colour-1 defects (2 B); coefficients from rho in registers
        per_launch = (16 if sor else 14) * N
        alg_total = kt_n * per_launch + (nv * 2 * N if sor and dopts.inner_nu1 > 0 else 0)
        kname = ("k_sweep_otf_fused (finest level, one whole red/black sweep, out of place, FP32, "
                 "coefficients from rho on the fly%s)" % (
                     ", over-relaxed omega=%.2f" % omega if sor else ""))
        tkey = "sweep_otf_fused_sor_fine" if sor else "sweep_otf_fused_fine"
    else:
        # one colour half-sweep a launch: the other colour's e (2 B) and both colours' rho (4 B)
        # read, the own colour's f read (2 B) and e written (2 B) = 10 B; over-relaxed also reads
        # the own colour's old e (2 B) = 12 B
        per_launch = (12 if sor else 10) * N
        # over-relaxed: the last pre-smoothing colour-1 half-sweep of each V-cycle also writes
        # its cells' defects (2 B per level cell) for the restriction
        alg_total = kt_n * per_launch + (nv * 2 * N if sor and dopts.inner_nu1 > 0 else 0)
        kname = ("k_gsrb_otf_staged (finest level, one colour half-sweep, FP32, coefficients "
                 "from rho on the fly%s)" % (", over-relaxed omega=%.2f" % omega if sor else ""))
        tkey = "gsrb_otf_staged_sor_fine" if sor else "gsrb_otf_staged_fine"
    avg_s = (kt_ms / kt_n) / 1e3 if kt_n else float("nan")
    alg_bytes = alg_total / kt_n if kt_n else float("nan")
    achieved = alg_bytes / avg_s / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            tj = json.load(f)
        ent = tj.get(tkey)
        if ent and ent.get("cells"):
            traffic = ent["dram_bytes_per_launch"] * N / ent["cells"]
    roofline = {"bound": "hbm", "kernel": kname,
                "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": traffic,
                "alg_bytes_per_launch": alg_bytes, "avg_launch_ms": avg_s * 1e3,
                "launches": kt_n, "peak_kind": peak_kind}
    cls_ms = {nm: sum(s["ktime_ms"][i] for s in st_mixed) / K for i, nm in enumerate(capi.KT_NAMES)}

    # ---- e2e through the public C ABI with pinned host fabs ---------------------------------
    e2e = None
    if not args.no_e2e:
        per = [b == capi.MAC_BC_PER for b in c.bc_lo]

        def pinned_like(a):
            t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
            v = t.numpy().reshape(a.shape, order="F")
            v[...] = a
            return t, v

        def fab_set():
            keep = []
            fu = []
            for d in range(c.dm):
                lst = []
                for f in lay.to_fabs(c.umac[d], ng=1, face_dir=d, periodic=per):
                    t, v = pinned_like(f)
                    keep.append(t)
                    lst.append(v)
                fu.append(lst)
            fr, fp, fs = [], [], []
            for f in lay.to_fabs(c.rho, ng=1, periodic=per):
                t, v = pinned_like(f)
                keep.append(t)
                fr.append(v)
            for f in lay.to_fabs(c.phi0, ng=1):
                t, v = pinned_like(f)
                keep.append(t)
                fp.append(v)
            for f in lay.to_fabs(c.macrhs, ng=0):
                t, v = pinned_like(f)
                keep.append(t)
                fs.append(v)
            return keep, fu, fr, fp, fs

        E = args.e2e_steps
        # two page-locked input sets used in turn; a set is refilled with the pristine inputs
        # (host copy, outside the timed calls) before it is used again
        sets = [fab_set() for _ in range(2)]
        pristine = fab_set()
        P = MacProjector(lay, c.dx, bc, precision="mixed", stream=stream.cuda_stream,
                         **inner_opts)
        nbytes = lambda lst: sum(x.nbytes for x in lst)  # noqa: E731
        s0 = sets[0]
        u_bytes = sum(nbytes(s0[1][d]) for d in range(c.dm))
        # host -> device: edge velocities, rho, rhs, phi guess, beta0; device -> host: edge
        # velocities and phi (whole fabs, ghosts included)
        h2d = u_bytes + nbytes(s0[2]) + nbytes(s0[4]) + nbytes(s0[3]) + 8 * (2 * c.n[-1] + 1)
        d2h = u_bytes + nbytes(s0[3])

        def refill(s):
            for d in range(c.dm):
                for a, b in zip(s[1][d], pristine[1][d]):
                    a[...] = b
            for a, b in zip(s[3], pristine[3]):
                a[...] = b

        for s in sets:   # warm-up: one call on each page-locked set (first use maps the pages)
            P.macproject(s[1], s[3], s[2], s[4], c.beta0, c.beta0_edge, strict=True)
            refill(s)
        step_s, dev_ms = [], []
        ck_e2e = Clocks(local, period_s=0.1)
        ck_e2e.start()
        for k in range(E):
            s = sets[(k + 1) % 2]
            barrier()
            t0 = time.perf_counter()
            st = P.macproject(s[1], s[3], s[2], s[4], c.beta0, c.beta0_edge, strict=True)
            barrier()
            step_s.append(time.perf_counter() - t0)
            dev_ms.append(round(st["setup_ms"] + st["solve_ms"], 3))
            refill(s)
        ck_e2e = ck_e2e.stop()
        secs = max_over_ranks(sum(step_s))
        P.close()
        link = link_rates(dev)
        link["h2d_ms_per_step"] = round(h2d / link["h2d_gbs"] / 1e6, 3)
        link["d2h_ms_per_step"] = round(d2h / link["d2h_gbs"] / 1e6, 3)
        e2e = {"value": world * E / secs, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "steps": E,
               "ms_per_step": [round(x * 1e3, 3) for x in step_s],
               "device_ms_per_step": dev_ms,
               "api": "mac_macproject (MAC_PTR_HOST; page-locked per-box fabs, 8 boxes of 128^3 "
                      "+ 1 ghost, copied by the copy engines on a transfer stream overlapped "
                      "with the setup and the copy-back)",
               "precision": "mixed", "clocks": ck_e2e, "link": link}

    # ---- CPU baseline: one full solve of the workload by the oracle (rank 0, N = 1) ---------
    cpu = None
    if not args.no_cpu and rank == 0 and world == 1:
        import oracle as O
        nlev = O.nlevels_for_boxes([c.box])
        threads = host_cores()
        t0 = time.perf_counter()
        _, _, sto = O.macproject(c.umac, c.phi0, c.rho, c.dx, c.bc_lo, c.bc_hi, macrhs=c.macrhs,
                                 beta0=c.beta0, beta0_edge=c.beta0_edge, nlevels=nlev,
                                 threads=threads)
        secs = time.perf_counter() - t0
        cpu = {"value": 1.0 / secs, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"one full {c.n[0]}^3 FP64 solve ({sto['vcycles']} V-cycles), "
                         f"C++/OpenMP restatement of MAESTRO macproject + FBoxLib MG"}

    # ---- the other configurations (rank 0, N = 1; after every timed region of the headline) ---
    configs = None
    if not args.no_configs and rank == 0 and world == 1:
        try:
            configs = measure_configs(dev, with_cpu=not args.no_cpu)
        except Exception as ex:   # reported in the line, the headline stands
            configs = {"error": repr(ex)[:400]}

    launches = sum(s["launches"] for s in st_mixed)
    rr = max(s["rel_resid"] for s in st_mixed)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
        "warmup": args.warmup, "ms_per_step": ms_mixed / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 V-cycles + f64 refinement",
        "data": "synthetic (seeded stratified atmosphere)",
        "config": mac_config(args.config, c.n, c.box, world),
        "precision": "mixed",
        "fp64": {"value": fp64_value, "unit": UNIT, "ms_per_step": ms_fp64 / K,
                 "vcycles": st_fp64[-1]["vcycles"], "rel_resid": st_fp64[-1]["rel_resid"]},
        "mixed_over_fp64": value / fp64_value,
        "mixed": {"refine_iters": st_mixed[-1]["refine_iters"],
                  "inner_vcycles": args.inner or capi.default_opts().inner_vcycles,
                  "inner_omega": capi.default_opts().inner_omega,
                  "adaptive_inner": not args.fixed_inner,
                  "inner_cycle": "V(%d,%d)" % (capi.default_opts().inner_nu1,
                                               capi.default_opts().inner_nu2),
                  "vcycles": st_mixed[-1]["vcycles"], "rel_resid": rr,
                  "phi_err_vs_fp64": phi_err, "u_err_vs_fp64": u_err,
                  "ms_by_class": cls_ms},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": ck_mixed,
        "clocks_fp64": ck_fp64,
        "configs": configs,
    }
    if rank == 0:
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
