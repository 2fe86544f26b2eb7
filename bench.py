"""Benchmark of the md_sim GB300 hot path: ns/day of the MD step on one GPU.

Default workload (the largest single-GPU system of the metric): bulk water, 32,768 rigid SPC/E-type
waters (98,304 atoms) in a 99.3 A periodic box, alpha 0.32, rcut 10 A, kmax 24 (29,038 k vectors),
dt 1 fs, synthetic and seeded (no public dataset exists for this path).  The interfacial slab
(2,048 waters between two oxide walls), the 8,192-water SHAKE system and the batch of 64 uneven
interfacial replicas run after it as extra lines (`other_configs`).

  value     ns/day of the resident MD step (move_predict, force_get, move_correct, SHAKE on the
            device), inputs resident in HBM; each of the K timed steps is bracketed by CUDA events
            on the library's stream and L2 is flushed (256 MB write) between steps.
  e2e       ns/day of the drop-in MD step a Fortran host makes: the Gear predictor on host arrays
            (mdg_host_predict on all host cores, the reference's move_predict), mdg_force_get
            with the host arrays pinned (positions host->device, forces, torques and energies back),
            the Gear corrector on the host (mdg_host_correct) and mdg_shake for surface atoms; the
            whole step is inside the timed region (host clock).
  roofline  dominant phase of the step, from mdg_phase_times (CUDA events), against the measured
            peak of its pipe.
  fp64_gpu  the plain FP64 form from the same start, its roofline against a measured FP64 rate
            (cuBLAS DGEMM through torch), and the mixed form's errors against it.
  cpu_baseline  the oracle (CPU restatement of the reference loops, OpenMP over all host cores,
            -O2 -ffast-math) on a bounded sample of the same workload.

--impl reference times that CPU implementation alone and prints its own line.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ns/day on 1 GB300: mixed+learned vs plain FP64 GPU at ΔF_rms≤1e-5; %roofline"
UNIT = "ns/day"
DEFAULT_CONFIG = "bulk32k"


def ns_per_day(sec_per_step, dt_fs=1.0):
    return 86400.0 / sec_per_step * dt_fs * 1e-6


# --------------------------------------------------------------------------------------------
def make_workload(name):
    from md_sim_gb300 import configs

    if name == "slab2048":
        s, prm = configs.slab_water()
        desc = ("interfacial slab: 2048 rigid SPC/E-type waters between two rocksalt (001) walls "
                "(3200 sites, q +-1.2 e, Buckingham wall-O), 42.1x42.1x84.2 A, EW3DC, alpha 0.30, "
                "rcut 10 A, kmax 10/knmax 20 (4338 k), dt 1 fs")
    elif name == "bulk256":
        s, prm = configs.bulk_water()
        desc = "bulk water: 256 rigid SPC/E-type waters, 19.73 A box, alpha 0.30, rcut 9, kmax 7 (775 k), dt 1 fs"
    elif name == "bulk32k":
        s, prm = configs.large_bulk_water()
        desc = ("large bulk water: 32768 rigid SPC/E-type waters (98304 atoms), 99.3 A periodic box, alpha 0.32, "
                "rcut 10 A, kmax 24 (29038 k), dt 1 fs")
    elif name == "shake8k":
        s, prm = configs.shake_water()
        desc = ("8192 SHAKE-constrained 3-site waters on rocksalt walls (19x19 cells, 11552 sites), "
                "tol 1e-10, dt 1 fs")
    elif name == "replicas64":
        s, prm = configs.replica_slabs(n=64)[0]
        desc = "first of the 64 uneven interfacial replicas (the CPU arm times one replica)"
    else:
        raise SystemExit(f"unknown config {name}")
    return s, prm, desc


def config_dict(name, desc, precision, args, s):
    """The `config` of a JSON line: identical for both arms apart from `precision`."""
    return {"workload": desc, "config": name, "precision": precision,
            "l2": "flushed (256 MB write) between timed GPU steps; inputs larger than L2 on the CPU arm",
            "equilibration_steps": args.equil,
            "ensemble": "NVE" if s.temper == -1.0 else f"NVT {s.temper} K"}


def host_cpu():
    """Host CPU model and the cores this process may use (lscpu, sched_getaffinity)."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.TimeoutExpired):
        pass
    try:
        cores = len(os.sched_getaffinity(0))
    except AttributeError:
        cores = os.cpu_count()
    return model, cores


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    def __init__(self, index=0):
        self.rows = []
        self.proc = None
        self.index = index

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
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
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for k, n in enumerate(names):
                if len(r) > 4 + k and r[4 + k].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0), "bf16_tflops": d.get("bf16_tflops", 1900.0),
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained", 1700.0), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "source": "fallback"}


def fp64_measured_tflops(torch, n=4096, reps=5):
    """FP64 rate of this GPU measured here: cuBLAS DGEMM (torch.matmul in float64, 2 n^3 flops),
    best of `reps`, CUDA events.  The denominator of the FP64 phases' roofline."""
    dev = torch.device("cuda", torch.cuda.current_device())
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) * 1e-3)
    del a, b
    return 2.0 * n ** 3 / best / 1e12


def site_pairs(s, ctx, rcut):
    """Accepted site pairs of one force evaluation: listed head pairs with head distance within rcut
    (molecular cutoff, src/forcem.f90:299) times the site products; plus head-wall site terms."""
    (li, lj), (wi, wj) = ctx.get_lists()
    t = s.itype - 1
    nsi = s.nsi[t]

    def acc(i, j, wall):
        i, j = i - 1, j - 1
        dx = s.x0[i] - s.x0[j]
        dy = s.y0[i] - s.y0[j]
        dz = s.z0[i] - s.z0[j]
        dx -= s.lx * np.round(dx / s.lx)
        dy -= s.ly * np.round(dy / s.ly)
        if ctx.prm.pbc_z_list and not wall:
            dz -= s.lz * np.round(dz / s.lz)
        ok = dx * dx + dy * dy + dz * dz <= rcut * rcut
        return int((nsi[i][ok] * (1 if wall else nsi[j][ok])).sum())

    return acc(li, lj, False), acc(wi, wj, True) if len(wi) else 0


def fp32_nominal_tflops():
    """152 SMs x 128 FP32 lanes x 2 flops x max SM clock (no measured FP32 peak on this machine)."""
    mhz = 2070.0
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        mhz = json.load(open(p)).get("sm_max_mhz", mhz)
    return 152 * 128 * 2 * mhz * 1e6 / 1e12


def roofline(ctx, s, prm, precision, pk, config_name="", fp64_peak=None):
    """Roofline of the dominant force phase (and of the reciprocal and pair phases), from CUDA-event
    phase times of mdg_phase_times and the algorithmic work per unit:
      pair phases   45 flops per accepted site pair (FP64 pipe, or FP32 + MUFU when mixed)
      reciprocal    18 flops per (atom, valid k) in FP64; 24 flops per (atom, valid k) for the
                    three complex products of the tensor-core form, whose ceiling is the dense
                    16-bit tensor peak / 3 (hi*hi + hi*lo + lo*hi).
    FP64 phases are set against the measured DGEMM rate (fp64_peak)."""
    from md_sim_gb300.abi import MDG_MIXED

    ph = ctx.phase_times(reps=5)
    nk = len(ctx.kvectors()[0])
    hh, hw = site_pairs(s, ctx, prm.rcut)
    mixed = precision == MDG_MIXED
    tf = os.path.join(ROOT, "profiles", "traffic.json")
    traffic_tab = json.load(open(tf)) if os.path.exists(tf) else {}
    fp64_src = "measured here: cuBLAS DGEMM 4096^3 through torch (float64)"

    def one(kind):
        t = ph[kind] * 1e-3
        if kind == "reciprocal":
            units = s.nmove * nk
            if mixed:
                flops, bound, peak, src = 24.0 * units, "tensor", pk["bf16_tflops"] / 3.0, pk["source"] + " bf16 burst /3"
            else:
                flops, bound, peak, src = 18.0 * units, "fp64", fp64_peak, fp64_src
        else:
            units = hh if kind == "pairs" else hw
            flops = 45.0 * units
            if mixed:
                bound, peak, src = "fp32", fp32_nominal_tflops(), "nominal FP32 (152 SM x 128 lanes x 2 x max clock)"
            else:
                bound, peak, src = "fp64", fp64_peak, fp64_src
        achieved = flops / max(t, 1e-12) / 1e12
        return {"bound": bound, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak if peak else None,
                "traffic": traffic_tab.get(f"{kind}:{'mixed' if mixed else 'fp64'}:{config_name}"),
                "traffic_unit": "DRAM bytes per launch (profiles/traffic.json, ncu)", "kernel": kind,
                "ms_per_launch": ph[kind], "units_per_launch": int(units), "flops_per_unit": flops / max(units, 1),
                "peak_source": src}

    dom = max(("pairs", "walls", "reciprocal"), key=lambda k: ph[k])
    out = one(dom)
    out["phase_ms"] = ph
    pairs = one("pairs")
    pairs["site_pairs_per_s"] = pairs["units_per_launch"] / max(ph["pairs"] * 1e-3, 1e-12)
    return out, one("reciprocal"), pairs


# --------------------------------------------------------------------------------------------
def cpu_reference(s, prm, sample_steps, threads=None, target_s=10.0, warmup=1):
    """CPU restatement of the reference (oracle, OpenMP) on a bounded sample: ns/day.  The
    sample grows to about target_s of CPU work after `warmup` untimed steps."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build as oracle_build

    from md_sim_gb300 import abi

    oracle_build.build()
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    lib = abi.Lib(oracle_build.path("libmdref_omp.so"), "ref_")
    s2 = s.copy()
    ctx = abi.Context(lib, s2, prm)
    ctx.set_state(s2)
    ctx.run(max(1, warmup))  # the first step includes lazy allocations
    t0 = time.perf_counter()
    ctx.run(sample_steps)
    dt = (time.perf_counter() - t0) / sample_steps
    n = int(min(2000, max(0, target_s / max(dt, 1e-9) - sample_steps)))
    if n > 0:
        t0 = time.perf_counter()
        ctx.run(n)
        dt = (time.perf_counter() - t0) / n
        sample_steps = n
    return ns_per_day(dt, s.dt), dt, sample_steps


def _barrier():
    """All ranks of a multi-GPU replica run meet here (no-op on one GPU)."""
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def time_resident(ctx, K, stream, flush, torch):
    """K resident steps, each bracketed by CUDA events on the library stream, L2 flushed between;
    under torchrun the ranks start and end the timed region together (barriers)."""
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    torch.cuda.synchronize()
    _barrier()
    with torch.cuda.stream(stream):
        for k in range(K):
            flush.zero_()
            ev[k][0].record(stream)
            ctx.run_async(1)
            ev[k][1].record(stream)
    stream.synchronize()
    torch.cuda.synchronize()
    _barrier()
    return [a.elapsed_time(b) for a, b in ev]


def nve_drift(ctx, s, nsteps, every=100):
    """Total energy htot (src/move.f90 bookkeeping) sampled every `every` resident steps over
    nsteps: relative change and least-squares slope per ns."""
    h = []
    done = 0
    t0 = time.perf_counter()
    while done < nsteps:
        rep = ctx.run(min(every, nsteps - done))
        done += min(every, nsteps - done)
        h.append((done, rep["htot"], rep["tempnow"]))
    wall = time.perf_counter() - t0
    t = np.array([x[0] for x in h], float) * s.dt * 1e-6  # ns
    e = np.array([x[1] for x in h], float)
    slope = float(np.polyfit(t, e, 1)[0]) if len(t) > 1 else 0.0
    return {"steps": int(nsteps), "dt_fs": s.dt, "htot_first": float(e[0]), "htot_last": float(e[-1]),
            "rel_change": float((e[-1] - e[0]) / abs(e[0])), "slope_per_ns": slope,
            "slope_per_ns_per_molecule": slope / max(s.nrig + s.ncons, 1),
            "temp_first": float(h[0][2]), "temp_last": float(h[-1][2]), "wall_s": wall,
            "unit": "htot in the reference's energy unit (kJ/mol)"}


def fp64_compare(lib, s_start, prm, args, stream, flush, torch, pk, fp64_peak, config_name):
    """Plain FP64 GPU form from the same equilibrated start (same timing), its roofline, and the
    mixed form's force / energy / pressure error against FP64 on that configuration."""
    import dataclasses

    from md_sim_gb300 import abi
    from md_sim_gb300.abi import MDG_FP64

    p64 = dataclasses.replace(prm, precision=MDG_FP64)
    fm = abi.Context(lib, s_start.copy(), prm)
    f64 = abi.Context(lib, s_start.copy(), p64)
    em, e64 = fm.force_get(s_start.copy()), f64.force_get(s_start.copy())
    fm.close()
    f64.close()
    d = em["f"] - e64["f"]
    err = {
        "dF_rms_rel": float(np.linalg.norm(d) / np.linalg.norm(e64["f"])),
        "dF_max_abs": float(np.abs(d).max()),
        "uconf_rel": float(abs(em["uconf"] - e64["uconf"]) / abs(e64["uconf"])),
        "uewa_rel": float(abs(em["uewa"] - e64["uewa"]) / max(abs(e64["uewa"]), 1e-300)),
        # the reference's pressure is the wall force per area (src/forcem.f90:1081); it never
        # accumulates a virial (vir is zeroed at src/forcem.f90:103), so press is the observable
        "press_abs": float(abs(em["press"] - e64["press"])),
        "press_rel": (float(abs(em["press"] - e64["press"]) / abs(e64["press"])) if e64["press"] != 0.0 else None),
    }
    s = s_start.copy()
    ctx = abi.Context(lib, s, p64)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_state(s)
    ctx.run(args.warmup)
    K = min(args.steps, args.fp64_steps)
    per_step = time_resident(ctx, K, stream, flush, torch)
    roof, roof_recip, roof_pairs = roofline(ctx, s, p64, MDG_FP64, pk, config_name, fp64_peak)
    ctx.close()
    t = float(np.sum(per_step)) / K * 1e-3
    return {"value": ns_per_day(t, s.dt), "unit": UNIT, "ms_per_step": t * 1e3, "steps": K,
            "error_vs_fp64": err, "roofline": roof, "roofline_reciprocal": roof_recip, "roofline_pairs": roof_pairs}


def _pinned_pool(lib, held, nbytes):
    """Host arrays carved from one region pinned in place through the library (as a Fortran host
    pins its module arrays once, mdg_pin_host).  Array starts are staggered by a varying number of
    cache lines: arrays that all began on 64 KB boundaries would share cache sets and slow the host
    integrator's streaming loops several-fold."""
    import mmap

    nbytes = -(-nbytes // 65536) * 65536
    mm = mmap.mmap(-1, nbytes)
    buf = np.frombuffer(mm, dtype=np.uint8)
    if lib.pin_host(buf.ctypes.data, nbytes) != 0:
        raise RuntimeError("mdg_pin_host failed: " + (lib.last_error(None) or b"").decode())
    held.append((buf, mm))
    state = {"off": 0, "k": 0}

    def alloc(n):
        off = -(-state["off"] // 64) * 64 + 64 * ((state["k"] * 17) % 64)
        end = off + 8 * max(n, 1)
        if end > nbytes:
            raise RuntimeError("pinned pool exhausted")
        state["off"], state["k"] = end, state["k"] + 1
        return buf[off:end].view(np.float64)[:n]

    return alloc


def e2e_arm(lib, s_start, prm, args, shake_model=None):
    """The drop-in MD step end to end: host predictor, mdg_force_get on the pinned host arrays,
    host corrector (+ mdg_shake), W untimed steps then K timed steps from the equilibrated start."""
    import ctypes as C

    from md_sim_gb300 import abi

    K = min(args.steps, args.e2e_steps)
    s = s_start.copy()
    held = []
    ctx = abi.Context(lib, s.copy(), prm)
    if shake_model is not None:
        ctx.set_shake_model(shake_model)  # the seed of the resident arm (mdg_shake_set_model)
    if args.autotune:
        ctx.set_state(s.copy())
        ctx.autotune(3)
    pool = 8 * (20 * s.ntota + 64 * max(s.nrig, 1) + 4 * s.nmove + 2 * s.nijt) + (1 << 20)
    hg = abi.HostGear(lib, s, alloc=_pinned_pool(lib, held, pool))
    a = hg.arr
    dp = abi._dp
    st = C.byref(a.st)
    fargs = ([dp(x) for x in a.x] + [dp(x) for x in a.c[0]] + [dp(x) for x in a.rs]
             + [dp(x) for x in hg.ft + hg.fc + hg.tq] + [None, None, None, C.byref(hg.e)])
    cargs = [dp(x) for x in hg.ft + hg.fc + hg.tq]
    shake = s.nmove > s.nliqa
    sargs = [dp(x) for x in a.x] + [dp(x) for x in a.old] + [dp(x) for x in hg.ft] + [None, C.byref(hg.tk),
                                                                                      C.byref(hg.sweeps)]
    predict, correct, force_get, shake_call = lib.host_predict, lib.host_correct, lib.force_get, lib.shake
    h, g, e = ctx.h, hg.h, hg.e
    tp, tf, tc, ts = [], [], [], []
    for k in range(args.warmup + K):
        t0 = time.perf_counter()
        rc = predict(g, st)
        t1 = time.perf_counter()
        rc = rc or force_get(h, *fargs)
        t2 = time.perf_counter()
        rc = rc or correct(g, st, *cargs, C.c_double(e.uconf))
        t3 = time.perf_counter()
        if rc == 0 and shake:
            rc = shake_call(h, *sargs)
        t4 = time.perf_counter()
        if rc != 0:
            raise RuntimeError(f"e2e step failed: {rc} {lib.last_error(ctx.h)}")
        if k >= args.warmup:
            tp.append(t1 - t0)
            tf.append(t2 - t1)
            tc.append(t3 - t2)
            ts.append(t4 - t3)
    rep = hg.report()
    ctx.close()
    hg.close()
    for arr, _ in held:
        lib.unpin_host(arr.ctypes.data)
    nm, nflex = s.nmove, s.nmove - s.nriga
    h2d = 8 * (6 * nm + 3 * s.nrig) + (8 * (3 * nm + 3 * (s.ntota - s.nliqa)) if shake else 0)
    d2h = 8 * (3 * nflex + 6 * s.nrig + 3 + 2 * s.nijt) + (8 * (3 * nm + 3 * (s.ntota - s.nliqa)) if shake else 0)
    step = np.array(tp) + np.array(tf) + np.array(tc) + np.array(ts)
    t = float(np.mean(step))
    return {"value": ns_per_day(t, s.dt), "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "path": ("drop-in MD step: mdg_host_predict (host cores, OpenMP) -> mdg_force_get -> mdg_host_correct"
                     + (" -> mdg_shake" if shake else "") + ", host arrays pinned once by mdg_pin_host"),
            "steps": K, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "host_integrator_ms": float(np.mean(tp) + np.mean(tc)) * 1e3, "force_call_ms": float(np.mean(tf)) * 1e3,
            "shake_call_ms": float(np.mean(ts)) * 1e3 if shake else 0.0, "tempnow_last": rep["tempnow"]}


def learned_arm(lib, ctx, s_start, args, K, stream, flush, torch, value, t_step):
    """The learned SHAKE seed on the same start and step count; returns (report, seeded per-step
    times, model)."""
    from md_sim_gb300 import learned

    t0 = time.perf_counter()
    w, how = learned.load_or_train(lib, ctx, s_start)
    t_model = time.perf_counter() - t0
    ctx.set_state(s_start.copy())
    sw_plain = learned.sweep_stats(ctx, 20)
    ctx.set_state(s_start.copy())
    ctx.set_shake_model(w)
    sw_seed = learned.sweep_stats(ctx, 20)
    ctx.set_state(s_start.copy())
    ctx.run(args.warmup)
    per_seed = time_resident(ctx, K, stream, flush, torch)
    ph_seed = ctx.phase_times(reps=5)
    ctx.set_shake_model(None)
    ph_plain = ctx.phase_times(reps=5)
    t_seed = float(np.sum(per_seed)) / K * 1e-3
    rep = {
        "model": how, "model_s": t_model,
        "value_plain_shake": value, "ms_per_step_plain_shake": t_step * 1e3,
        "value_seeded": ns_per_day(t_seed, s_start.dt), "ms_per_step_seeded": t_seed * 1e3,
        "sweeps_per_molecule_plain": sw_plain.mean_sweeps, "sweeps_per_molecule_seeded": sw_seed.mean_sweeps,
        "max_sweeps_plain": sw_plain.max_sweeps, "max_sweeps_seeded": sw_seed.max_sweeps,
        "shake_ms_plain": ph_plain["shake"], "shake_ms_seeded": ph_seed["shake"],
        "tolerance": ctx.prm.shake_tol2,
    }
    return rep, per_seed, w


def widom_arm(ctx, s, args):
    """Widom insertions (chempot) on the context's last force evaluation: wall time per call on the
    GPU (host clock around mdg_widom: generator on the host, one kernel, results back)."""
    from md_sim_gb300 import abi

    seed0 = 14135621772.0
    band = (1.0, min(6.0, 0.45 * s.lw))
    f = abi.MDG_WIDOM_SKIP_OVERLAP
    ctx.widom(16, band[0], band[1], 8, 4, seed0, flags=f)  # warm-up: scratch and attributes
    t0 = time.perf_counter()
    r = ctx.widom(args.widom, band[0], band[1], 8, 4, seed0, flags=f)
    t_gpu = time.perf_counter() - t0
    return {"insertions": args.widom, "band_A": list(band), "orientations": int(r["inave"].sum()),
            "ms_per_call": t_gpu * 1e3, "orientations_per_s": r["inave"].sum() / t_gpu,
            "flags": "skip overlapping positions"}


def run_workload(lib, name, args, torch, stream, flush, pk, fp64_peak, headline=True):
    """One workload: the resident mixed-precision step (with the learned seed where there are
    SHAKE molecules), its rooflines, the FP64 form from the same start, and the drop-in e2e step.
    The headline workload adds the drift run and the CPU baseline."""
    from md_sim_gb300 import abi, configs
    from md_sim_gb300.abi import MDG_FP64, MDG_MIXED

    s, prm, desc = make_workload(name)
    precision = MDG_MIXED if args.precision == "mixed" else MDG_FP64
    prm.precision = precision
    ctx = abi.Context(lib, s, prm)
    ctx.set_stream(stream.cuda_stream)
    configs.equilibrate(ctx, s, steps=args.equil, every=20)
    s_start = s.copy()
    ctx.set_state(s)
    tuning = ctx.autotune(5) if args.autotune else None
    ctx.run(args.warmup)
    K = args.steps
    with ClockSampler() as clk:
        per_step = time_resident(ctx, K, stream, flush, torch)
    rep = ctx.check()
    t_step = float(np.sum(per_step)) / K * 1e-3
    value = ns_per_day(t_step, s.dt)
    kps = ctx.kernels_per_step()
    ctx.get_state(s)
    roof, roof_recip, roof_pairs = roofline(ctx, s, prm, precision, pk, name, fp64_peak)
    learned_rep, shake_model = None, None
    if s.ncons > 0 and args.learned and precision == MDG_MIXED:
        learned_rep, per_seed, shake_model = learned_arm(lib, ctx, s_start, args, K, stream, flush, torch, value,
                                                         t_step)
        value, t_step, per_step = learned_rep["value_seeded"], learned_rep["ms_per_step_seeded"] * 1e-3, per_seed
    drift = nve_drift(ctx, s, args.drift) if (headline and args.drift > 0) else None
    widom = widom_arm(ctx, s, args) if (args.widom > 0 and s.nwall > 0) else None
    ctx.close()
    cmp64 = None
    if precision == MDG_MIXED and args.fp64_steps > 0:
        cmp64 = fp64_compare(lib, s_start, prm, args, stream, flush, torch, pk, fp64_peak, name)
        cmp64["speedup"] = value / cmp64["value"]
    e2e = e2e_arm(lib, s_start, prm, args, shake_model)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": K, "warmup": args.warmup,
        "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if precision == MDG_FP64 else "f32 pairs + f16x3 tensor reciprocal (f64 state)",
        "data": "synthetic (seeded)",
        "config": config_dict(name, desc, args.precision, args, s),
        "e2e": e2e,
        "gpu_launches": int(kps * K),
        "kernels_per_step": kps,
        "tuning": tuning,
        "roofline": roof,
        "roofline_reciprocal": roof_recip,
        "roofline_pairs": roof_pairs,
        "clocks": clk.summary(),
        "step_report": {k: rep[k] for k in ("tempnow", "htot", "uconf", "rebuilds", "steps")},
        "step_ms_min_median_max": [min(per_step), float(np.median(per_step)), max(per_step)],
    }
    if cmp64 is not None:
        out["fp64_gpu"] = cmp64
    if learned_rep is not None:
        out["learned_shake"] = learned_rep
    if drift is not None:
        out["nve_drift"] = drift
    if widom is not None:
        out["widom"] = widom
    if headline and args.cpu_baseline:
        v, dt, n = cpu_reference(s, prm, args.cpu_steps)
        model, cores = host_cpu()
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "cpu": model, "kind": "port",
                               "sample": f"{n} MD steps of the same workload after one untimed step "
                                         f"({dt * 1e3:.2f} ms/step), OpenMP over {cores} host cores"}
    return out


def _summary(o):
    """Compact record of an extra workload's line."""
    keep = {"value": o["value"], "unit": o["unit"], "ms_per_step": o["ms_per_step"], "config": o["config"],
            "e2e": {k: o["e2e"][k] for k in ("value", "ms_per_step", "host_integrator_ms", "force_call_ms")},
            "roofline_reciprocal": {k: o["roofline_reciprocal"][k] for k in ("achieved", "peak", "frac", "ms_per_launch")},
            "roofline_pairs": {k: o["roofline_pairs"][k] for k in ("achieved", "peak", "frac", "ms_per_launch")},
            "kernels_per_step": o["kernels_per_step"], "clocks": o["clocks"]}
    if "fp64_gpu" in o:
        f = o["fp64_gpu"]
        keep["fp64_gpu"] = {"value": f["value"], "speedup": f["speedup"], "error_vs_fp64": f["error_vs_fp64"]}
    for k in ("learned_shake", "widom"):
        if k in o:
            keep[k] = o[k]
    return keep


def replica_extra(args, arm):
    """Config 4 as an extra line beside the single systems: the batch arm's compact record, or its
    error (the headline line is printed either way)."""
    try:
        o = arm(args)
        return {k: o[k] for k in ("value", "unit", "ms_per_step", "config", "per_replica_ns_per_day", "sequential",
                                  "batch_speedup_vs_sequential", "batch_mode", "step_ms_min_median_max", "clocks")}
    except Exception as e:  # noqa: BLE001
        return {"error": f"{type(e).__name__}: {e}"}


def gpu_arm(args):
    import torch

    import md_sim_gb300

    lib = md_sim_gb300.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    pk = peaks()
    fp64_peak = fp64_measured_tflops(torch)
    out = run_workload(lib, args.config, args, torch, stream, flush, pk, fp64_peak, headline=True)
    out["fp64_peak_tflops_measured"] = fp64_peak
    extras = [c for c in args.extra.split(",") if c and c != args.config]
    if extras:
        out["other_configs"] = {}
        for name in extras:
            if name == "replicas64":
                out["other_configs"][name] = replica_extra(args, replicas_arm)
                continue
            o = run_workload(lib, name, args, torch, stream, flush, pk, fp64_peak, headline=False)
            out["other_configs"][name] = _summary(o)
    return out


def replica_partition(n, rank, world):
    """Replicas of this rank: r, r + world, r + 2 world, ... (every replica on exactly one rank)."""
    return list(range(rank, n, world))


def replicas_arm(args, rank=0, world=1):
    """Config 4: uneven interfacial replicas stepped together by one graph launch per batch step
    (mdg_batch), timed with CUDA events on the batch stream; against the same replicas stepped one
    after another with their own graphs.  Under torchrun rank r takes the replicas r, r + world, ..."""
    import torch

    import md_sim_gb300
    from md_sim_gb300 import abi, configs
    from md_sim_gb300.abi import MDG_FP64, MDG_MIXED

    lib = md_sim_gb300.load()
    n = args.replicas
    t0 = time.perf_counter()
    allsys = configs.replica_slabs(n=n)  # built in full on every rank: the seeds run in sequence
    systems = [allsys[i] for i in replica_partition(n, rank, world)]
    t_build = time.perf_counter() - t0
    precision = MDG_MIXED if args.precision == "mixed" else MDG_FP64
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    ctxs = []
    t0 = time.perf_counter()
    for s, prm in systems:
        prm.precision = precision
        c = abi.Context(lib, s, prm)
        c.set_state(s)
        ctxs.append(c)
    t_create = time.perf_counter() - t0
    # untimed: each replica's start-up transient with velocity rescaling, as for the single systems
    # (without it the synthetic starts heat up for hundreds of steps)
    t0 = time.perf_counter()
    for c, (s, _) in zip(ctxs, systems):
        configs.equilibrate(c, s, steps=args.equil, every=20)
    t_equil = time.perf_counter() - t0
    t0 = time.perf_counter()
    tunings = [c.autotune(3) for c in ctxs] if args.autotune else []
    t_tune = time.perf_counter() - t0
    batch = abi.Batch(lib, ctxs)
    batch.set_stream(stream.cuda_stream)
    batch.set_mode(abi.MDG_BATCH_PHASES if args.batch_mode == "phases" else abi.MDG_BATCH_GRAPHS)
    batch.run(args.warmup)                # untimed: graph build and warm-up
    # The thinnest films (a few hundred waters on the widest walls) heat up by several hundred K
    # per 100 steps under NVE even after the rescaled start (the oracle's own dynamics do the
    # same), and a few leave the stable range after about 500 steps: at most 200 timed steps.
    K = min(args.steps, 200)
    with ClockSampler() as clk:
        per_step = []
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
        torch.cuda.synchronize()
        _barrier()
        with torch.cuda.stream(stream):
            for k in range(K):
                flush.zero_()
                ev[k][0].record(stream)
                batch.run_async(1)
                ev[k][1].record(stream)
        stream.synchronize()
        _barrier()
        per_step = [a.elapsed_time(b) for a, b in ev]
    for c in ctxs:
        c.check()
    t_batch = float(np.sum(per_step)) / K * 1e-3
    phased = batch.phased()
    # the other graph form of the same batch, for comparison (untimed warm-up, then Ko steps)
    other = "graphs" if args.batch_mode == "phases" else "phases"
    batch.set_mode(abi.MDG_BATCH_GRAPHS if other == "graphs" else abi.MDG_BATCH_PHASES)
    batch.run_async(3)
    torch.cuda.synchronize()
    Ko = max(5, K // 4)
    eo = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(Ko)]
    with torch.cuda.stream(stream):
        for k in range(Ko):
            flush.zero_()
            eo[k][0].record(stream)
            batch.run_async(1)
            eo[k][1].record(stream)
    stream.synchronize()
    t_other = float(np.sum([a.elapsed_time(b) for a, b in eo])) / Ko * 1e-3
    for c in ctxs:
        c.check()
    batch.close()  # the replicas step alone again with their own plans
    # the same replicas one after another, each with its own graph, on the same stream
    for c in ctxs:
        c.set_stream(stream.cuda_stream)
        c.run_async(1)
    torch.cuda.synchronize()
    Ks = max(5, K // 10)
    a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        flush.zero_()
        a_.record(stream)
        for _ in range(Ks):
            for c in ctxs:
                c.run_async(1)
        b_.record(stream)
    stream.synchronize()
    t_seq = a_.elapsed_time(b_) * 1e-3 / Ks
    for c in ctxs:
        c.check()
    atoms = int(sum(s.ntota for s, _ in systems))
    waters = int(sum(s.nrig for s, _ in systems))
    dt = systems[0][0].dt
    nloc = len(systems)
    value = ns_per_day(t_batch, dt) * nloc
    return {
        "metric": METRIC + " (config 4: replica batch)", "value": value, "unit": "replica-ns/day",
        "n_gpus": 1, "steps": K, "warmup": args.warmup, "ms_per_step": t_batch * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if precision == MDG_FP64 else "f32 pairs + f16x3 tensor reciprocal (f64 state)",
        "data": "synthetic (seeded)",
        "config": {"workload": f"{n} interfacial replicas, waters U{{500..4000}}, walls 7-14+ cells, one graph launch "
                               f"per batch step; this rank: {nloc} replicas, {waters} waters, {atoms} sites",
                   "config": "replicas64", "precision": args.precision, "l2": "flushed (256 MB write) between timed steps",
                   "equilibration_steps": args.equil, "ensemble": "NVE"},
        "replicas_this_rank": nloc,
        "per_replica_ns_per_day": ns_per_day(t_batch, dt),
        "sequential": {"ms_per_step": t_seq * 1e3, "value": ns_per_day(t_seq, dt) * nloc, "unit": "replica-ns/day",
                       "how": "each replica's own graph, one after another on one stream"},
        "batch_speedup_vs_sequential": t_seq / t_batch,
        "batch_mode": {"timed": args.batch_mode, "replicas_in_batched_loops": phased,
                       other: {"ms_per_step": t_other * 1e3, "value": ns_per_day(t_other, dt) * nloc,
                               "steps": Ko}},
        "setup_s": {"build": t_build, "create": t_create, "equilibration": t_equil, "autotune": t_tune},
        "tuning": _tuning_summary(tunings),
        "clocks": clk.summary(),
        "step_ms_min_median_max": [min(per_step), float(np.median(per_step)), max(per_step)],
    }


def _tuning_summary(tunings):
    """Per-replica autotuner choices folded into counts, with the summed force time before/after."""
    if not tunings:
        return None
    choice = {}
    for key in ("pair_blocks", "tc_rows_per_cta"):
        for t in tunings:
            k = f"{key}={t[key]}"
            choice[k] = choice.get(k, 0) + 1
    splits = [t["tc_atom_splits"] for t in tunings]
    return {"choices": choice, "tc_atom_splits_min_max": [min(splits), max(splits)],
            "force_ms_sum_before": float(sum(t["ms_before"] for t in tunings)),
            "force_ms_sum_after": float(sum(t["ms_after"] for t in tunings))}


def _allreduce(x, op):
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=op)
    return float(t.item())


def aggregate_ranks(out, world):
    """Replicas only: every rank ran its own independent system(s) on its own GPU with no exchange.
    The slowest rank's step time (max over ranks) sets the pace; the job's value is the replicas
    of all ranks at that pace.  A single-system workload runs one replica per rank."""
    import torch.distributed as dist

    ms = _allreduce(out["ms_per_step"], dist.ReduceOp.MAX)
    nloc = out.get("replicas_this_rank", 1)
    ntot = int(round(_allreduce(nloc, dist.ReduceOp.SUM)))
    per = out["value"] / nloc * out["ms_per_step"] / ms  # one replica's ns/day at the slowest pace
    out = dict(out)
    if isinstance(out.get("e2e"), dict) and "value" in out["e2e"]:
        e = _allreduce(out["e2e"]["value"], dist.ReduceOp.MIN)  # the slowest rank's drop-in steps
        out["e2e"] = dict(out["e2e"], value=e * world)
    if "gpu_launches" in out:
        out["gpu_launches"] = int(round(_allreduce(out["gpu_launches"], dist.ReduceOp.SUM)))
    out["replica_value"] = per
    out["replicas_total"] = ntot
    out["value"] = per * ntot
    out["ms_per_step"] = ms
    out["n_gpus"] = world
    out["scaling"] = "weak"
    out["config"] = dict(out["config"], parallelism=f"replicas over {world} GPUs (independent systems, no collective)")
    return out


def reference_arm(args):
    """The reference's own CPU path on the host cores: the oracle port (the Fortran reference has
    no compiler on this machine or the GPU machine), OpenMP over every host core, W untimed and K timed
    MD steps of the same workload and config as the GPU arm (fewer only if K steps would pass
    about four minutes; the line says so)."""
    from md_sim_gb300.abi import MDG_FP64

    s, prm, desc = make_workload(args.config)
    prm.precision = MDG_FP64
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build as oracle_build

    from md_sim_gb300 import abi

    oracle_build.build()
    model, cores = host_cpu()
    os.environ["OMP_NUM_THREADS"] = str(cores)
    lib = abi.Lib(oracle_build.path("libmdref_omp.so"), "ref_")
    s2 = s.copy()
    t0 = time.perf_counter()
    ctx = abi.Context(lib, s2, prm)
    ctx.set_state(s2)
    t_init = time.perf_counter() - t0
    W = max(1, args.warmup)
    t0 = time.perf_counter()
    ctx.run(W)
    t_w = (time.perf_counter() - t0) / W
    K = args.steps
    capped = False
    if K * t_w > 240.0:
        K = max(3, int(240.0 / t_w))
        capped = True
    t0 = time.perf_counter()
    ctx.run(K)
    t = (time.perf_counter() - t0) / K
    v = ns_per_day(t, s.dt)
    sample = (f"{K} MD steps after {W} untimed (CPU restatement of the reference loops, OpenMP over {cores} host "
              f"cores; the Fortran reference has no compiler here; create {t_init:.1f} s untimed)")
    if capped:
        sample += f"; {args.steps} steps requested, capped to about four minutes of CPU time"
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 1, "steps": K,
            "warmup": W, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "impl": "reference",
            "config": config_dict(args.config, desc, "fp64", args, s),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "cpu": model, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def profile_run(args):
    """Minimal command for ncu: the steps run last, after create and two warm-up steps."""
    import md_sim_gb300
    from md_sim_gb300 import abi
    from md_sim_gb300.abi import MDG_FP64, MDG_MIXED

    lib = md_sim_gb300.load()
    if args.config == "replicas64":
        return profile_batch(args, lib)
    s, prm, desc = make_workload(args.config)
    prm.precision = MDG_MIXED if args.precision == "mixed" else MDG_FP64
    ctx = abi.Context(lib, s, prm)
    ctx.set_state(s)
    ctx.run(2)
    ctx.run_async(args.steps)
    rep = ctx.check()
    print(json.dumps({"profile_steps": args.steps, "kernels_per_step": ctx.kernels_per_step(),
                      "tempnow": rep["tempnow"]}))


def profile_batch(args, lib):
    """Replica batch for ncu: create, one checked batch step per graph form, then one step in phase
    order inside the NVTX range "phases" and one as child graphs inside "graphs"."""
    import torch

    from md_sim_gb300 import abi, configs

    ctxs = []
    for s, prm in configs.replica_slabs(n=args.replicas):
        prm.precision = abi.MDG_MIXED
        c = abi.Context(lib, s, prm)
        c.set_state(s)
        ctxs.append(c)
    batch = abi.Batch(lib, ctxs)
    out = {"profile_steps": 1, "replicas": len(ctxs)}
    for name, mode in (("phases", abi.MDG_BATCH_PHASES), ("graphs", abi.MDG_BATCH_GRAPHS)):
        batch.set_mode(mode)
        batch.run(1)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push(name)
        batch.run_async(1)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        out[name + "_phased"] = batch.phased()
    for c in ctxs:
        c.check()
    batch.close()
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default=DEFAULT_CONFIG,
                    choices=["slab2048", "bulk256", "bulk32k", "shake8k", "replicas64"])
    ap.add_argument("--extra", default="slab2048,shake8k,replicas64",
                    help="workloads measured after the headline one, as compact lines (empty: none)")
    ap.add_argument("--replicas", type=int, default=64)
    ap.add_argument("--batch-mode", choices=("phases", "graphs"), default="phases",
                    help="replica batch graph form: real-space loops of all replicas in one kernel each "
                         "(phases) or every replica's own step graph as a child graph (graphs)")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--fp64-steps", type=int, default=20,
                    help="steps of the plain FP64 GPU comparison arm (0 = skip)")
    ap.add_argument("--equil", type=int, default=200)
    ap.add_argument("--drift", type=int, default=10000,
                    help="NVE energy drift over this many extra resident steps of the headline workload (0 = skip)")
    ap.add_argument("--no-learned", dest="learned", action="store_false",
                    help="skip the learned SHAKE seed arm (workloads with SHAKE only)")
    ap.add_argument("--widom", type=int, default=2000,
                    help="Widom insertion positions timed on the final state (0 = skip; wall systems only)")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="keep the default launch parameters instead of timing candidates (mdg_autotune)")
    ap.add_argument("--e2e-steps", type=int, default=60)
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--profile", action="store_true",
                    help="profiling run: create, 2 warm-up steps, then --steps resident steps, no extras")
    args = ap.parse_args()
    if args.profile:
        profile_run(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(reference_arm(args)))
        return
    if world > 1:
        # replicas only: every rank runs its own independent system(s) on its own GPU
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group(backend="nccl")
        args.cpu_baseline = False  # the CPU baseline is rank 0's at one GPU only
        args.extra = ""
    if args.config == "replicas64":
        out = replicas_arm(args, rank, world)
    else:
        out = gpu_arm(args)
    if world > 1:
        out = aggregate_ranks(out, world)
    if rank == 0:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
