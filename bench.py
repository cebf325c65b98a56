"""Benchmark of the coupled LBM-DEM time step (one GB300, replicas for N>1).

Workload (default): coupled sedimentation, 128^3 D3Q19 TRT in a no-slip box, seeded
non-overlapping spheres r ~ U[4,6] (random sequential addition from seed 2 until it
jams; the achieved count is reported), density ratio 2.5, gravity 1e-5, linear
spring-dashpot contacts (kn=1e3, e=0.8, mu=0.5), multiStep 3, populations FP32
(deviation storage) with FP64 DEM.  A "step" is one whole cycle: DEM substeps, coupling
masks, fused collide+stream, element force reduction.

value      MLUPS over the active nodes (inside-particle nodes included, as the
           reference counts activeNodes), device-resident, graph-replayed cycles: the
           median of windows of --steps cycles that, with the end-to-end windows
           between them, run the configuration's whole 5000-cycle job (the suspension
           settles and its contacts grow, so later cycles cost more: early_value is the
           rate of the windows that start in the first 200 cycles).
e2e        same metric through the C-ABI per step with host buffers: hb_set_body_force
           and hb_cycle(1) every step, the body force going in as graph kernel parameters
           and the element state and hydrodynamic forces coming out into page-locked
           mapped host arrays (hb_set_element_sink), timed until the last step's state
           is on the host.
roofline   the fused collide+stream kernel: algorithmic bytes per launch / its
           CUDA-event duration, against the measured HBM copy bandwidth.
cpu_baseline  the CPU oracle (this repository's C++ restatement of the reference, the
           reference itself cannot be built on the aarch64 GPU host) on a bounded
           sample of the same workload.
fp64_form  the same workload with FP64 populations: step time, FP32 speed-up, and the
           FP32 form's velocity (relative L2, L-inf) and density error against it after
           --compare-steps cycles from the same initial state.
adjoint    drag adjoint on the 96^3 channel with 64 fixed spheres (FP32, 2000 steps,
           checkpoints every 100): device time per step of forward + reverse, and dJ/dtau
           against central differences of the FP64 forward.
configs    MLUPS of configurations 1, 3 and 4 (channel FP64; dam break FP32; 256^3 with
           16000 spheres in FP32 and FP16 storage).

Multi-GPU: the path does not shard on one box; --gpus N runs N independent replicas
(one per rank, no collective), value = sum over ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

B_LU = {0: 2 * 19 * 8 + 1, 1: 2 * 19 * 4 + 1, 2: 2 * 19 * 2 + 1}  # bytes per lattice update
DTYPE = {0: "f64", 1: "f32", 2: "f16-storage/f32-compute"}


def workload(precision, deposited=False):
    """Configuration 2 (hybird_gb300.workloads.sedimentation): 128^3 TRT, seeded RSA
    spheres r ~ U[4, 6] from seed 2 (1514 placed before the packing jams); deposited=True
    drops the same spheres onto the floor, so that every sphere is in contact."""
    from hybird_gb300.workloads import sedimentation
    return sedimentation(precision, deposited=deposited)


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        cmd = ["nvidia-smi", f"--id={self.index}",
               "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
               "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
               "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "50"]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([s.strip() for s in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[0]))
                mx = float(s[1])
                for k, nm in enumerate(names):
                    if s[3 + k].lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def cpu_sample(params, spheres, steps, threads):
    """CPU oracle on a bounded sample of the workload: one untimed cycle, then `steps`
    timed whole cycles.  Returns the rate, the timed seconds, the cycles run and the
    oracle's final node types, density and velocity (the checker of the GPU forms'
    error on the same cycles)."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    from oracle_port import OracleSim
    o = OracleSim(params, spheres, threads=threads)
    active = int(o.lib.hbo_active(o.h))
    o.cycle(1)  # first cycle includes the neighbour rebuild; not timed
    t0 = time.perf_counter()
    o.cycle(steps)
    dt = time.perf_counter() - t0
    lat = o.lattice()
    o.close()
    return active * steps / dt / 1e6, dt, steps + 1, {k: lat[k] for k in ("type", "n", "u")}


def error_vs_oracle(p32, spheres, cycles, ref):
    """Velocity (relative L2, L-inf relative to max |u|) and density (absolute L-inf)
    error of the GPU's FP32, FP16-storage and FP64 forms against the oracle's state
    `ref` after the same `cycles` whole cycles from the same initial state."""
    from hybird_gb300 import abi
    from hybird_gb300.gpu import GpuSim
    act = (ref["type"] == 0) | (ref["type"] == 3)
    u0 = ref["u"].reshape(3, -1)[:, act]
    out = {"cycles": cycles}
    for name, prec in (("f32", abi.HB_FP32), ("f16s", abi.HB_FP16S), ("f64", abi.HB_FP64)):
        p = abi.HbParams.from_buffer_copy(p32)
        p.precision = prec
        g = GpuSim(p, spheres)
        g.cycle(cycles)
        l = g.lattice(("type", "n", "u"))
        g.close()
        du = l["u"].reshape(3, -1)[:, act] - u0
        out[name] = {"u_rel_l2": float(np.sqrt((du ** 2).sum() / (u0 ** 2).sum())),
                     "u_rel_linf": float(np.abs(du).max() / np.abs(u0).max()),
                     "rho_abs_linf": float(np.abs(l["n"][act] - ref["n"][act]).max()),
                     "types_identical": bool(np.array_equal(l["type"], ref["type"]))}
    return out


def dem_loaded(steps):
    """The DEM contact path under load: configuration 2 with the spheres deposited on
    the floor and on each other (every sphere in contact from the start; multiStep 10,
    at which such a bed is stable), FP32 populations, FP64 DEM.  Whole-cycle time, the cooperative DEM kernel's phases from
    device timestamps, candidate pairs and overlapping contacts of the last substep."""
    from hybird_gb300 import abi
    from hybird_gb300.gpu import GpuSim
    p, spheres = workload(abi.HB_FP32, deposited=True)
    g = GpuSim(p, spheres)
    g.cycle(5)
    ms, ms_lb, _ = g.time_cycles(steps)
    ph = g.profile_phases(max(5, steps // 4))
    st = g.status()
    g.close()
    ms_step = ms / steps
    multi = p.multi_step
    dem_us = float(ph[:1 + 2 * multi].sum())  # element forces + the substeps
    return {"workload": "configuration 2 spheres deposited on the floor (%d spheres), FP32 populations, "
                        "FP64 DEM, multiStep %d" % (len(spheres), multi),
            "ms_per_step": round(ms_step, 4), "lattice_kernel_ms": round(ms_lb, 4),
            "contacts_last_substep": st.contacts, "candidate_pairs": st.pairs,
            "pairs_evaluated_per_s": round(st.pairs * multi / (ms_step * 1e-3), 1),
            "contacts_per_s": round(st.contacts * multi / (ms_step * 1e-3), 1),
            "dem_kernel_us": round(dem_us, 2),
            "phases_us": [round(float(v), 2) for v in ph]}


def fp64_compare(p32, spheres, steps):
    """The FP64 form of the same workload: its step time, and the FP32 and FP16-storage
    forms' velocity and density errors against it after `steps` cycles from the same
    initial state."""
    from hybird_gb300 import abi
    from hybird_gb300.gpu import GpuSim
    p64 = abi.HbParams.from_buffer_copy(p32)
    p64.precision = abi.HB_FP64
    p16 = abi.HbParams.from_buffer_copy(p32)
    p16.precision = abi.HB_FP16S
    out = {"steps": steps}
    lat = {}
    for name, p in (("f64", p64), ("f32", p32), ("f16s", p16)):
        g = GpuSim(p, spheres)
        if name == "f64":
            g.cycle(3)
            ms, _, _ = g.time_cycles(10)
            out["ms_per_step_f64"] = ms / 10
            g.close()
            g = GpuSim(p, spheres)
        g.cycle(steps)
        l = g.lattice()
        lat[name] = {k: l[k] for k in ("type", "n", "u")}
        g.close()
    act = (lat["f64"]["type"] == 0) | (lat["f64"]["type"] == 3)
    u64 = lat["f64"]["u"].reshape(3, -1)[:, act]
    du = lat["f32"]["u"].reshape(3, -1)[:, act] - u64
    out["u_rel_l2"] = float(np.sqrt((du ** 2).sum() / (u64 ** 2).sum()))
    out["u_rel_linf"] = float(np.abs(du).max() / np.abs(u64).max())
    out["rho_abs_linf"] = float(np.abs(lat["f32"]["n"][act] - lat["f64"]["n"][act]).max())
    d16 = lat["f16s"]["u"].reshape(3, -1)[:, act] - u64
    out["fp16s"] = {"u_rel_l2": float(np.sqrt((d16 ** 2).sum() / (u64 ** 2).sum())),
                    "u_rel_linf": float(np.abs(d16).max() / np.abs(u64).max()),
                    "rho_abs_linf": float(np.abs(lat["f16s"]["n"][act] - lat["f64"]["n"][act]).max())}
    return out


def config_rates(steps):
    """MLUPS of the other configurations (graph-replayed cycles, active nodes at the start):
    1 = 64x32x32 periodic channel, BGK FP64; 3 = dam break 256x128x128 with free surface,
    Bingham, Smagorinsky and 500 spheres (FP32); 4 = 256^3 with 16000 spheres (FP32 and
    FP16-storage)."""
    from hybird_gb300 import abi
    from hybird_gb300.gpu import GpuSim
    from hybird_gb300.workloads import channel, dam_break, precision_box
    out = {}
    from hybird_gb300.workloads import sedimentation
    p_mbb, s_mbb = sedimentation(abi.HB_FP32)
    p_mbb.coupling = abi.HB_MOVING_BB
    cases = [("c1_channel_64x32x32_bgk_f64", channel(precision=abi.HB_FP64), None),
             ("c2_moving_bounce_back_f32", p_mbb, s_mbb),
             ("c3_dambreak_256x128x128_f32", *dam_break(abi.HB_FP32)),
             ("c4_256cube_16000_spheres_f32", *precision_box(abi.HB_FP32)),
             ("c4_256cube_16000_spheres_f16s", *precision_box(abi.HB_FP16S))]
    for name, p, spheres in cases:
        g = GpuSim(p, spheres)
        l0 = g.lattice(("type", "inside"))
        act = (l0["type"] == 0) | (l0["type"] == 3)
        A = int(act.sum())
        g.cycle(5)
        ms, ms_lb, _ = g.time_cycles(steps)
        g.close()
        out[name] = {"mlups": round(A / (ms / steps * 1e-3) / 1e6, 1), "ms_per_step": round(ms / steps, 4),
                     "lattice_kernel_ms": round(ms_lb, 4), "active_nodes": A,
                     "spheres": 0 if spheres is None else len(spheres)}
        if p.coupling == abi.HB_MOVING_BB:  # the nodes inside particles are solid in this mode
            F = int((act & (l0["inside"] == 0)).sum())
            out[name]["fluid_nodes"] = F
            out[name]["mlups_fluid_nodes"] = round(F / (ms / steps * 1e-3) / 1e6, 1)
    return out


def adjoint_measure(steps):
    """Drag adjoint on 96^3 (64 fixed spheres r=6, TRT tau 0.7, FP32, body force 2e-6,
    inlet/outlet planes): device time per step of forward + reverse (checkpoints every
    100 steps, segments recomputed), and dJ/dtau against central differences of the FP64
    forward (relative step 1e-4)."""
    from hybird_gb300 import abi
    from hybird_gb300.gpu import GpuSim
    from hybird_gb300.workloads import adjoint_channel
    p, obj, uin = adjoint_channel(precision=abi.HB_FP32)
    g = GpuSim(p, None, obj)
    F = tuple(p.lbF)
    g.adjoint_drag(steps, 0.7, F, uin, abi.HB_FP32, 100)  # allocation and warm-up
    J, dF, dtau, duin = g.adjoint_drag(steps, 0.7, F, uin, abi.HB_FP32, 100)
    ms_f, ms_r, nf, nr = g.adjoint_timing()
    h = 1e-4 * 0.7
    fd = (g.adjoint_forward(steps, 0.7 + h, F, uin, abi.HB_FP64, 100)
          - g.adjoint_forward(steps, 0.7 - h, F, uin, abi.HB_FP64, 100)) / (2 * h)
    g.close()
    return {"workload": "96^3 channel, 64 fixed spheres r=6, TRT tau 0.7, F=2e-6, inlet/outlet u0=0.02, FP32",
            "steps": steps, "checkpoint_every": 100, "ms_forward": round(ms_f, 3), "ms_reverse": round(ms_r, 3),
            "ms_per_step": round((ms_f + ms_r) / steps, 5), "forward_steps": nf, "reverse_steps": nr,
            "J": J, "dJ_dtau": dtau, "dJ_dtau_fd_fp64": fd, "dJ_dtau_rel_err": abs(dtau - fd) / abs(fd)}


def run_reference(args, rank):
    """The reference arm: the reference's CPU algorithm (the oracle port; the reference
    sources do not travel to the GPU host) on this machine's host cores, on the same workload,
    metric and unit: min(W, 3) untimed cycles, then min(K, 200) timed cycles."""
    from hybird_gb300 import abi
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(REPO, "tests"))
    from oracle_port import OracleSim
    p, spheres = workload(abi.HB_FP64)
    threads = os.cpu_count() or 1
    steps = max(1, min(args.steps, 200))
    warm = max(1, min(args.warmup, 3))
    o = OracleSim(p, spheres, threads=threads)
    active = int(o.lib.hbo_active(o.h))
    o.cycle(warm)
    t0 = time.perf_counter()
    o.cycle(steps)
    dt = time.perf_counter() - t0
    o.close()
    v = active * steps / dt / 1e6
    line = {"impl": "reference", "metric": "MLUPS (coupled LBM-DEM step)", "value": round(v, 3),
            "unit": "MLUPS", "n_gpus": args.gpus, "steps": steps, "warmup": warm,
            "ms_per_step": round(dt / steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "coupled sedimentation 128^3 D3Q19 TRT, %d spheres r~U[4,6], multiStep 3"
                       % len(spheres), "lattice": [128, 128, 128], "spheres": len(spheres)},
            "cpu_baseline": {"value": round(v, 3), "unit": "MLUPS", "cores": threads, "kind": "port",
                             "sample": f"{steps} whole cycles after {warm} untimed cycles ({dt:.1f} s)"},
            "e2e": {"value": round(v, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def lattice_traffic(prec):
    """DRAM bytes per launch of the lattice kernel from the committed ncu capture of this
    workload (profiles/), or None."""
    try:
        with open(os.path.join(REPO, "profiles", "lattice_kernel_traffic.json")) as fh:
            d = json.load(fh)
        return d["dram_bytes_per_launch"].get({0: "f64", 1: "f32", 2: "f16s"}[prec])
    except (OSError, KeyError, ValueError):
        return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp64", "fp32", "fp16s"])
    ap.add_argument("--cpu-steps", type=int, default=100, help="0 skips the CPU baseline")
    ap.add_argument("--compare-steps", type=int, default=100,
                    help="cycles of the FP64 form run beside the FP32 one (speed-up and error)")
    ap.add_argument("--adjoint-steps", type=int, default=2000, help="0 skips the adjoint measurement")
    ap.add_argument("--config-steps", type=int, default=50,
                    help="timed cycles of configurations 1, 3 and 4 (0 skips them)")
    ap.add_argument("--dem-steps", type=int, default=40,
                    help="timed cycles of the deposited (all spheres in contact) workload (0 skips it)")
    ap.add_argument("--min-cycles", type=int, default=2500,
                    help="device windows of --steps cycles are repeated until this many cycles ran "
                         "(as many run in the end-to-end windows between them: 2500 covers the "
                         "5000-cycle job of the configuration); the median window is reported")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    from hybird_gb300.replicas import Replicas
    rep = Replicas()
    rank, world, local = rep.rank, rep.world, rep.local
    if args.impl == "reference":
        run_reference(args, rank)
        rep.close()
        return

    import ctypes as C
    from hybird_gb300 import abi
    from hybird_gb300.gpu import GpuSim, check, lib

    os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
    prec = {"fp64": abi.HB_FP64, "fp32": abi.HB_FP32, "fp16s": abi.HB_FP16S}[args.precision]
    p, spheres = workload(prec)
    g = GpuSim(p, spheres)
    st = g.status()
    L = lib()
    # active nodes and inside-particle nodes from the device state
    gl = g.lattice()
    act = (gl["type"] == 0) | (gl["type"] == 3)
    A = int(act.sum())
    A_in = int((act & (gl["inside"] == 1)).sum())
    del gl
    # warm-up
    for _ in range(args.warmup):
        check(L.hb_cycle(g.h, 1))
    check(L.hb_synchronize(g.h))
    rep.barrier()
    # Timed windows of exactly K cycles, repeated until --min-cycles ran; the median
    # window is reported.  Each device-resident window (inputs larger than L2:
    # 2 x 19 x 2.1M x 4 B = 319 MB of populations) is followed by an end-to-end window of
    # K steps through the C-ABI with host buffers, so both are measured at the same state
    # of the settling suspension: every step the host sets the body force (24 B, carried
    # into the cycle graph as kernel parameters) and runs one cycle, whose last kernel
    # writes the element state a host driver reads (x0, x1, FHydro, MHydro) into
    # page-locked mapped host arrays (hb_set_element_sink); an end-to-end window ends when
    # the last step's state has landed on the host.  The lattice mirror is off in these
    # windows, as it is in the device windows: no step writes the node fields that only a
    # lattice download would read.
    E = g.E
    host = np.zeros((4, 3 * E))
    check(L.hb_host_register(host.ctypes.data_as(C.c_void_p), host.nbytes))
    force = np.array(p.lbF[:], dtype=np.float64)
    ptr = [host[k].ctypes.data_as(C.c_void_p) for k in range(4)]
    windows = max(1, -(-args.min_cycles // args.steps))
    per_step, per_lb, e2e_step = [], [], []
    with Clocks(local) as clk:
        for _ in range(windows):
            ms_tot, ms_lb, kpc = g.time_cycles(args.steps)
            per_step.append(ms_tot / args.steps)
            per_lb.append(ms_lb)
            check(L.hb_set_element_sink(g.h, ptr[0], ptr[1], None, None, ptr[2], ptr[3],
                                        None, None, None, None, None))
            check(L.hb_set_lattice_mirror(g.h, 0))  # the driver reads element state only
            check(L.hb_synchronize(g.h))
            t0 = time.perf_counter()
            for _ in range(args.steps):
                check(L.hb_set_body_force(g.h, force.ctypes.data_as(C.c_void_p)))
                check(L.hb_cycle(g.h, 1))
            check(L.hb_synchronize(g.h))
            e2e_step.append((time.perf_counter() - t0) / args.steps)
            check(L.hb_set_lattice_mirror(g.h, 1))
            check(L.hb_set_element_sink(g.h, *([None] * 11)))
    check(L.hb_host_unregister(host.ctypes.data_as(C.c_void_p)))
    assert np.isfinite(host).all() and np.abs(host[2]).max() > 0.0
    k_med = int(np.argsort(per_step)[len(per_step) // 2])
    ms_step = rep.max(per_step[k_med])
    ms_lb = per_lb[k_med]
    value = rep.aggregate_rate(A, ms_step * 1e-3) / 1e6
    # the device windows that start in the first 200 cycles (device and end-to-end windows
    # alternate, so window w starts at cycle 2 w K after the warm-up)
    early = [v for w, v in enumerate(per_step) if 2 * w * args.steps < 200]
    early_value = rep.aggregate_rate(A, rep.max(float(np.mean(early))) * 1e-3) / 1e6
    e2e_dt = rep.max(float(np.median(e2e_step)))
    e2e = rep.aggregate_rate(A, e2e_dt) / 1e6
    e2e_steps = args.steps * windows
    # roofline of the fused kernel
    peak, peak_kind = measured_peak()
    bytes_launch = A * B_LU[prec] + A_in * (4 + 3 * (8 if prec == abi.HB_FP64 else 4))
    achieved = bytes_launch / (ms_lb * 1e-3) / 1e9 if ms_lb > 0 else None
    st = g.status()
    g.close()
    fp64 = fp64_compare(p, spheres, args.compare_steps) if args.compare_steps > 0 and prec != abi.HB_FP64 else None
    loaded = dem_loaded(args.steps) if args.dem_steps > 0 else None
    adj = adjoint_measure(args.adjoint_steps) if args.adjoint_steps > 0 else None
    cfgs = config_rates(args.config_steps) if args.config_steps > 0 else None
    step_bytes = bytes_launch  # the lattice kernel's algorithmic bytes are the step's bytes
    line = {
        "metric": "MLUPS (coupled LBM-DEM step)", "value": round(value, 2), "unit": "MLUPS",
        "early_value": round(early_value, 2),
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": DTYPE[prec], "data": "synthetic",
        "config": {"workload": "coupled sedimentation 128^3 D3Q19 TRT, %d spheres r~U[4,6], multiStep 3, "
                               "populations %s, DEM f64" % (E, args.precision),
                   "lattice": [128, 128, 128], "active_nodes": A, "inside_nodes": A_in, "spheres": E,
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (319 MB populations per step)",
                   "kernels_per_cycle": kpc, "timed_windows": windows,
                   "window_ms_per_step": [round(v, 4) for v in per_step]},
        "gpu_launches": kpc * args.steps,
        "e2e": {"value": round(e2e, 2), "unit": "MLUPS", "h2d_bytes_per_step": 24,
                "d2h_bytes_per_step": 4 * 3 * E * 8, "steps": e2e_steps,
                "window_ms_per_step": [round(v * 1e3, 4) for v in e2e_step]},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1) if achieved else None,
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4) if achieved else None,
                     "traffic": lattice_traffic(prec), "kernel": "k_collide_stream_dev" if prec != abi.HB_FP64 else "k_collide_stream", "kernel_ms": round(ms_lb, 5),
                     "peak_kind": peak_kind, "bytes_per_launch": bytes_launch,
                     "step_frac": round(step_bytes / (ms_step * 1e-3) / 1e9 / peak, 4)},
        "clocks": clk.summary(),
        # candidate pairs are evaluated every substep; contacts/s at the last substep's count
        "dem": {"contacts_last_substep": st.contacts, "candidate_pairs": st.pairs,
                "pairs_evaluated_per_s": round(st.pairs * p.multi_step / (ms_step * 1e-3), 1),
                "contacts_per_s": round(st.contacts * p.multi_step / (ms_step * 1e-3), 1)},
    }
    if loaded:
        line["dem_loaded"] = loaded
    if fp64:
        fp64["fp32_speedup"] = round(fp64.pop("ms_per_step_f64") / ms_step, 2)
        line["fp64_form"] = fp64
    if adj:
        line["adjoint"] = adj
    if cfgs:
        line["configs"] = cfgs
    if rank == 0 and args.cpu_steps > 0:
        threads = os.cpu_count() or 1
        try:
            p64, sph = workload(abi.HB_FP64)
            v, dt, ncyc, ref = cpu_sample(p64, sph, args.cpu_steps, threads)
            line["cpu_baseline"] = {"value": round(v, 3), "unit": "MLUPS", "cores": threads, "kind": "port",
                                    "sample": f"{args.cpu_steps} whole cycles of the same workload in FP64 "
                                              f"after one untimed cycle ({dt:.1f} s)"}
            # the GPU forms against this oracle run (same workload, same cycles)
            line["error_vs_oracle"] = error_vs_oracle(p, sph, ncyc, ref)
        except Exception as exc:  # noqa: BLE001
            line["cpu_baseline"] = {"value": None, "error": str(exc)[:200]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    rep.close()


if __name__ == "__main__":
    main()
