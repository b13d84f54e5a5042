"""Benchmark of the GB300 split-step propagator on the 256x256x2048 multipass-cell workload.

One bench step = one pass of the cell (Cav = 0.5 m at 400 fixed split steps per pass, mirror
lens at the end of the pass): 400 split steps over the 256x256x2048 complex64 field held in
HBM.  value = grid-point-steps/s = Nx*Ny*Nt*400*K / (device time of K passes), timed with CUDA
events on the stream the kernels run on, after W warm-up passes; the 1 GiB field is larger
than L2, so no flush is needed between passes.  e2e = the same metric through the public C
ABI with host buffers: every step uploads the complex128 field from pinned host memory
(mpc_field_upload), runs the pass (mpc_run_fixed) and downloads it (mpc_field_download).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--workload W]

--workload picks another cell for its own line (default cell256, the headline above): cell64 is
the 64x64x512 cell (0.2 mJ, one bench step = one pass of 200 fixed split steps), cell512 the
512x512x1024 plasma-dominated cell (3 mJ, 120 fs, argon 3 bar) under adaptive step doubling at
a local-error tolerance of 1e-5 (one bench step = 10 attempts of 3 split steps each; value counts
the split steps executed, `accepted_pt_steps_per_s` the accepted ones).

--impl reference times the reference's CPU path for this workload -- the FP64 restatement in
oracle/ (the reference's own FFTW/MPI build cannot be compiled; only plasma.c and a few
propagation.c functions build, see oracle/build_ref.sh) -- with OpenMP on all host cores, each
step a bounded sample of one split step of the same 256x256x2048 cell.
Multi-GPU: the cells of a sweep are independent, so N > 1 runs N independent replicas
(one cell per rank, no collective on the data path) and reports the aggregate.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

FALLBACK_HBM_GBS = 6800.0
METRIC = "grid-point-steps/s"
BYTES_PER_PT_STEP = 32  # two compulsory complex64 sweeps (read + write) per split step
FP64_NOMINAL_TFLOPS = 1.25  # GB300 FP64 vector rate, nominal


def fft_flop_per_pt_step(Nx: int, Ny: int, Nt: int) -> float:
    """FFT work of one split step per grid point at 5 n log2(n) per transform: three Nt-point
    t transforms (the self-steepening derivative, to time, back) and four x / y transforms."""
    import math
    return 3 * 5 * math.log2(Nt) + 2 * 5 * math.log2(Nx) + 2 * 5 * math.log2(Ny)


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def profile_traffic(names):
    """dram bytes per launch of a sweep from the committed ncu summaries of its kernels (summed
    over the kernels of the sweep), or None when one is missing."""
    total = 0.0
    for name in names:
        path = os.path.join(ROOT, "profiles", name)
        if not os.path.exists(path):
            return None
        val = None
        with open(path) as f:
            for ln in f:
                if ln.startswith("traffic_bytes_per_launch:"):
                    val = float(ln.split(":", 1)[1])
        if val is None:
            return None
        total += val
    return total


WORKLOADS = {
    "cell256": dict(cell="cell256", adaptive=False, per_step=400, cpu_steps=5,
                    desc="multipass cell 256x256x2048, fixed split steps, lens mirror, SST + ADK + plasma on",
                    step="one pass of the cell = 400 split steps",
                    profile={"pencil": ["pencil_step_256x256x2048.txt"],
                             "plane": ["plane_y_tma_256x256x2048.txt", "plane_x_tma_256x256x2048.txt"]}),
    "cell64": dict(cell="cell64", adaptive=False, per_step=200, cpu_steps=100,
                   desc="multipass cell 64x64x512, fixed split steps, lens mirror, SST + ADK + plasma on",
                   step="one pass of the cell = 200 split steps", profile=None),
    "cell512": dict(cell="cell512", adaptive=True, per_step=10, cpu_steps=2,
                    desc="plasma-dominated cell 512x512x1024 (3 mJ, 120 fs, argon 3 bar), adaptive step "
                         "doubling at 1e-5, lens mirror, SST + ADK + plasma on",
                    step="10 step-doubling attempts = 30 split steps", profile=None),
}


def make_workload(name: str = "cell256"):
    from mpc_gb300 import inputs
    cfg = getattr(inputs, WORKLOADS[name]["cell"])()
    p, A = inputs.make_cell(cfg)
    return cfg, p, A


def cpu_baseline_run(p, A, nsteps: int, threads: int, keep: bool = False):
    """The FP64 CPU restatement (oracle/) on `nsteps` split steps of the same cell: the time,
    and with keep the resulting field as well."""
    import oracle
    oracle.set_threads(threads)
    o = oracle.Oracle(p)
    B = A.copy()
    o.calibrate(B)
    st = o.new_state()
    t = time.perf_counter()
    o.run_fixed(B, st, nsteps)
    dt = time.perf_counter() - t
    return (dt, B) if keep else dt


def _power_spectrum(A, p):
    import torch
    F = torch.fft.fft(torch.from_numpy(A.reshape(p.Nt, p.Ny * p.Nx)).cuda(), dim=0)
    return (F.abs() ** 2).sum(dim=1).cpu().numpy()


def accuracy_of(p, A, ref, nsteps: int, variant: int) -> dict:
    """The device path's relative L2 errors after `nsteps` split steps from the same seeded,
    calibrated field, against the FP64 oracle's field `ref` (the CPU baseline's own run)."""
    from mpc_gb300 import capi
    with capi.Propagator(p.copy(variant=variant)) as prop:
        prop.upload(A, calibrate=True)
        prop.run_fixed(nsteps)
        got = prop.download()
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))  # noqa: E731
    out = {"split_steps": nsteps, "against": "FP64 oracle (CPU), same seeded input",
           "field_rel_l2": rel(got, ref), "spectrum_rel_l2": rel(_power_spectrum(got, p), _power_spectrum(ref, p))}
    whole = whole_run_accuracy(p)
    if whole:
        out["whole_run"] = whole
    return out


def whole_run_accuracy(p):
    """The whole run's errors against the FP64 GPU oracle from the committed report, if any."""
    path = os.path.join(ROOT, "profiles", f"accuracy_whole_run_{p.Nx}x{p.Ny}x{p.Nt}.txt")
    if not os.path.exists(path):
        return None
    out = {"source": os.path.relpath(path, ROOT)}
    with open(path) as f:
        for ln in f:
            for key in ("split_steps", "field_rel_l2", "spectrum_rel_l2", "energy_drift"):
                if ln.startswith(key + ":"):
                    out[key] = float(ln.split(":", 1)[1])
    return out


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return rank, world, local, dist
    return rank, world, local, None


def run_reference(args):
    rank, world, local, dist = dist_init()
    if rank != 0:
        if dist:
            dist.barrier()
        return
    wl = WORKLOADS[args.workload]
    cfg, p, A = make_workload(args.workload)
    cores = os.cpu_count() or 1
    times = []
    for i in range(args.warmup + args.steps):
        dt = cpu_baseline_run(p, A, 1, cores)
        if i >= args.warmup:
            times.append(dt)
    per = float(np.mean(times))
    value = p.N * 1 / per
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "grid-point-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": per * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Gaussian pulse + 1e-4 noise, argon 1 bar)",
            "config": {"workload": wl["desc"], "grid": [p.Nx, p.Ny, p.Nt],
                       "sample": "1 split step per bench step (CPU time bound)"},
            "cpu_baseline": {"value": value, "unit": "grid-point-steps/s", "cores": cores, "kind": "port",
                             "sample": f"1 split step of the {p.Nx}x{p.Ny}x{p.Nt} cell per bench step, FP64, OpenMP"},
            "e2e": {"value": value, "unit": "grid-point-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()


def run_gb300(args):
    rank, world, local, dist = dist_init()
    import torch
    torch.cuda.set_device(local)
    from mpc_gb300 import capi
    wl = WORKLOADS[args.workload]
    cfg, p, A = make_workload(args.workload)
    prop = capi.Propagator(p.copy(variant=args.variant))   # -1: the autotuner picks the kernel variant
    vinfo = prop.variant_info()
    # pinned host field for the end-to-end path (physical units, calibrated)
    pin = capi.PinnedArray(p.N)
    pin.array[:] = A
    prop.upload(pin.array, calibrate=True)
    prop.sync()
    pin.array[:] = prop.download()
    stream = torch.cuda.ExternalStream(prop.stream_handle())

    accepted = [0]

    def one_pass():
        if wl["adaptive"]:
            for _ in range(wl["per_step"]):
                accepted[0] += 1 - prop.step_double()["bad"]
        else:
            prop.run_fixed(wl["per_step"])

    for _ in range(args.warmup):
        one_pass()
    prop.sync()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    launches0 = prop.launch_count()
    accepted[0] = 0
    ev0.record(stream)
    for _ in range(args.steps):
        one_pass()
    ev1.record(stream)
    ev1.synchronize()
    launches = prop.launch_count() - launches0
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    torch.cuda.synchronize()
    if dist:
        t = torch.tensor([ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    split_steps = (3 if wl["adaptive"] else 1) * wl["per_step"] * args.steps
    value = p.N * split_steps * world / (ms / 1e3)
    accepted_rate = p.N * accepted[0] * world / (ms / 1e3)

    # per-sweep device time over one extra pass (events around every launch)
    prop.profile(True)
    one_pass()
    kt = prop.kernel_times()
    prop.profile(False)
    hbm, src = peaks()
    sweeps = {"pencil": (kt["pencil_ms"], kt["n_pencil"]), "plane": (kt["plane_ms"], kt["n_plane"])}
    dom = max(sweeps, key=lambda k: sweeps[k][0])
    dom_ms = sweeps[dom][0] / max(1, sweeps[dom][1])
    # one complex64 read + write of the whole field per kernel; the plane sweep of the two-pass
    # variants is two kernels (column strips, then row strips)
    passes = (2 if vinfo.get("PL", 1) >= 2 else 1) if dom == "plane" else 1
    bytes_launch = 16.0 * p.N * passes
    achieved = bytes_launch / (dom_ms / 1e3) / 1e9
    traffic = profile_traffic(wl["profile"][dom]) if wl["profile"] else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "traffic": traffic, "kernel": f"{dom} sweep",
                "peak_source": src, "per_sweep_ms": {k: v[0] / max(1, v[1]) for k, v in sweeps.items()},
                "step_frac_of_32B_floor": (value / world) * BYTES_PER_PT_STEP / (hbm * 1e9)}

    # end to end through the C ABI with host buffers
    e2e_steps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        prop.upload(pin.array)
        one_pass()
        prop.download(pin.array)
    e2e_s = time.perf_counter() - t0
    # where the end-to-end time goes: one more step with the stream drained after each phase
    t1 = time.perf_counter()
    prop.upload(pin.array)
    prop.sync()
    t2 = time.perf_counter()
    one_pass()
    prop.sync()
    t3 = time.perf_counter()
    prop.download(pin.array)
    t4 = time.perf_counter()
    phase = {"upload_ms": (t2 - t1) * 1e3, "steps_ms": (t3 - t2) * 1e3, "download_ms": (t4 - t3) * 1e3}
    e2e_split = (3 if wl["adaptive"] else 1) * wl["per_step"] * e2e_steps
    e2e = {"value": p.N * e2e_split * world / e2e_s, "unit": "grid-point-steps/s",
           "h2d_bytes_per_step": 16 * p.N, "d2h_bytes_per_step": 16 * p.N, "phases_one_step": phase}

    # the reference-signature drop-in: mpc_ssfmprop on a host field (pinned), one split step per
    # call with the complex128 field copied in and out every call, as MPC.c's loop would call it
    dropin = None
    if not wl["adaptive"]:
        st0 = prop.state()
        prop.ssfmprop(pin.array, p.dzz, 1, 0.0, p.puls_e)
        prop.sync()
        ncall = 5
        t0 = time.perf_counter()
        for _ in range(ncall):
            prop.ssfmprop(pin.array, p.dzz, 1, 0.0, p.puls_e)
        dt_call = (time.perf_counter() - t0) / ncall
        prop.set_state(st0)
        dropin = {"value": p.N * world / dt_call, "unit": "grid-point-steps/s", "ms_per_split_step": dt_call * 1e3,
                  "api": "mpc_ssfmprop on a pinned host complex128 field, one split step per call",
                  "h2d_bytes_per_step": 16 * p.N, "d2h_bytes_per_step": 16 * p.N}

    cpu = None
    accuracy = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        nst = wl["cpu_steps"]  # about 10 s on 16 host cores
        dt, Bref = cpu_baseline_run(p, A, nst, cores, keep=True)
        cpu = {"value": p.N * nst / dt, "unit": "grid-point-steps/s", "cores": cores, "kind": "port",
               "sample": f"{nst} split steps of the {p.Nx}x{p.Ny}x{p.Nt} cell, FP64 oracle/ restatement, OpenMP"}
        if not wl["adaptive"]:
            accuracy = accuracy_of(p, A, Bref, nst, args.variant)
        del Bref
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    fp32_peak = nsm * 128 * 2 * (clk.get("sm_mhz") or 2070.0) * 1e6 / 1e12
    fft_tflops = (value / world) * fft_flop_per_pt_step(p.Nx, p.Ny, p.Nt) / 1e12
    fft_rate = {"flop_per_pt_step": fft_flop_per_pt_step(p.Nx, p.Ny, p.Nt), "tflops": fft_tflops,
                "fp32_peak_tflops": fp32_peak, "frac_fp32": fft_tflops / fp32_peak,
                "fp64_nominal_tflops": FP64_NOMINAL_TFLOPS, "ratio_to_fp64": fft_tflops / FP64_NOMINAL_TFLOPS}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "grid-point-steps/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
                "data": "synthetic (seeded Gaussian pulse + 1e-4 noise, argon 1 bar)",
                "config": {"workload": wl["desc"], "step": wl["step"], "grid": [p.Nx, p.Ny, p.Nt],
                           "split_steps_per_step": split_steps // args.steps,
                           "l2": ("field > L2, no flush" if 8 * p.N > 129e6 else
                                  "field fits L2: the bench step's passes re-read it from L2"),
                           "parallelism": f"replicas x{world}", "kernel_variant": vinfo},
                "roofline": roofline, "fft_rate": fft_rate, "cpu_baseline": cpu, "e2e": e2e,
                "dropin": dropin, "accuracy": accuracy, "gpu_launches": launches, "clocks": clk}
        if wl["adaptive"]:
            line["accepted_pt_steps_per_s"] = accepted_rate
        print(json.dumps(line), flush=True)
    prop.close()
    pin.free()
    if dist:
        dist.barrier()


def run_profile_case(nsteps: int, variant: int = 0, workload: str = "cell256", all_kernels: bool = False):
    """A short target for ncu: upload the workload's field and run `nsteps` split steps,
    with no timing.  Launch order: the entry pencil sweep (template mode 0), then per split
    step one pencil sweep (mode 2) and one plane sweep.  With all_kernels, then every other
    kernel of the library once: one step-doubling attempt (k_richardson,
    k_pencil_energy_slots, k_beam_profiles), the diagnostics (pencil mode 5, k_spec), the
    step-size features (k_moments), the controller network's inference, loss gradient and one
    training epoch (k_mlp_predict, k_mlp_grad, k_adam), and the allocation-free nonlinear step
    (k_nonlinear_noalloc) on a complex64 copy of the field."""
    from mpc_gb300 import capi
    cfg, p, A = make_workload(workload)
    with capi.Propagator(p.copy(variant=variant)) as prop:
        prop.upload(A, calibrate=True)
        B = prop.download() if all_kernels else None   # the calibrated field, for the noalloc step
        prop.run_fixed(nsteps)
        prop.sync()
        if all_kernels:
            prop.step_double()
            prop.diag()
            prop.features()
            prop.sync()
        print(json.dumps({"profile_case": nsteps, "grid": [p.Nx, p.Ny, p.Nt], "launches": prop.launch_count()}))
    if all_kernels:
        import torch
        from mpc_gb300 import dzlearn
        mlp = dzlearn.load()
        rng = np.random.default_rng(0)
        X = rng.standard_normal((4096, capi.NFEATURES)).astype(np.float32)
        y = rng.standard_normal(4096).astype(np.float32)
        mlp.predict(X)
        mlp.loss_grad(X, y)
        mlp.train(X, y, epochs=1, batch=256)
        mlp.close()
        if p.Nt <= 2048:
            dev = torch.from_numpy(B.astype(np.complex64)).to("cuda")
            rc = capi.nonlinear_noalloc(p, dev.data_ptr(), p.dzz, torch.cuda.current_stream().cuda_stream)
            torch.cuda.synchronize()
            print(json.dumps({"noalloc_status": rc}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="cell256", choices=sorted(WORKLOADS))
    ap.add_argument("--variant", type=int, default=-1,
                    help="kernel variant of the grid (-1: autotune; pin one for profiler runs, whose "
                         "serialised timings mislead the autotuner)")
    ap.add_argument("--profile-case", type=int, default=0, metavar="NSTEPS",
                    help="run NSTEPS split steps of the workload and exit (an ncu target)")
    ap.add_argument("--all-kernels", action="store_true",
                    help="with --profile-case: then launch every other kernel of the library once")
    args = ap.parse_args()
    if args.profile_case:
        run_profile_case(args.profile_case, max(args.variant, 0), args.workload, args.all_kernels)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
