"""Benchmark of the batched mixed-precision CSP (models/s) on GB300.

Workload (one step = one batch): the mixed-precision batched CSP at B = 65536 models: weights over 107 ages x 12
metallicities per model, split-BF16 contraction with a 1284 x 5994 SSP basis (nebular lines in the young SSPs),
power-law dust (tau_V uniform 0-3), redshift uniform 0-6 with the Madau IGM, velocity smoothing sigma uniform
50-300 km/s, 40 filters; seeded synthetic inputs (libopensps_gb300.workloads.mixed_csp).

* ``value``: models/s with the inputs resident in HBM (opensps_gb300_batch_device), timed with CUDA events on the
  library's stream over ``--steps`` batches after ``--warmup`` (the 673 MB FP64 weight input of a step is larger than
  L2, so no flush is needed between steps).
* ``e2e``: the same through the OpenSPS C API (opensps_context_compute_csp_batch_grad with ssp_weights_z, no
  cotangents) from pinned host buffers: the weights and per-model parameters are copied in and the magnitudes,
  masses and L_bol copied out inside the timed region.
* ``roofline``: the contraction kernel (split-BF16 tcgen05 GEMM with its fused epilogue): 3 x 2 K P B executed
  bf16 FLOPs per launch over its mean CUDA-event duration, against the measured sustained bf16 peak.
* ``adjoint``: the reverse pass (compute_csp_batch_grad_rows) at B = 16384 with cotangents on 40 magnitudes and
  512 spectral bins, through the C API from page-locked host buffers (wall time), with its device stage times.
* ``ssp_operator``: the IMF-free batch through the SSP operator (a Kroupa IMF per model) at B = 1024, through the C
  API, with its device stage times.
* ``fp64_path`` / ``mixed_over_fp64``: the same workload through the plain FP64 GPU path (DGEMM age sums, every
  later stage in FP64) at B = 65536, and the mixed path's device models/s over it.
* ``cpu_baseline`` / ``--impl reference``: the FP64 CPU oracle (a restatement of OpenSPS's compute_csp_batch,
  the reference being Fortran with no compiler in this image) with OpenMP on all host cores, on a bounded sample.

With ``--gpus N`` under torchrun each rank runs its own batch (replicas: the models of different ranks are
independent; no collective on the data path) and ``value`` is the models of all ranks over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

K_AGES, N_Z, N_PIX = 107, 12, 5994
METRIC = "CSP models/s at B=65536: mixed vs FP64 at <=1e-4 rel; emulator speedup @0.01 mag"
WORKLOAD = ("mixed-precision batched CSP (split-BF16 contraction 1284x5994, nebular lines, power-law dust, "
            "Madau IGM z 0-6, velocity smoothing 50-300 km/s, 40 filters)")


def _peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"],
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained", d["bf16_tflops"]), "src": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "src": "fallback"}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    def __init__(self, path: Path):
        self.path = path
        self.proc = None

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200", "-i", str(int(os.environ.get("LOCAL_RANK", "0")))],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_oracle_rate(n_sample: int, seed: int = 5) -> dict:
    """The FP64 CPU oracle on n_sample models of the workload: models/s on all host cores."""
    from libopensps_gb300 import synthdata, workloads
    from oracle.oracle import Oracle
    o = Oracle(synthdata.load(), nbands=40)
    wz, params = workloads.mixed_csp(n_sample, seed=seed)
    o.csp_batch({k: v[:8] for k, v in params.items()}, wz[:8])   # warm
    t0 = time.perf_counter()
    o.csp_batch(params, wz)
    dt = time.perf_counter() - t0
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": n_sample / dt, "unit": "models/s", "cores": cores, "kind": "port", "seconds": dt,
            "sample": f"{n_sample} models of the B=65536 workload (FP64 oracle, OpenMP), {dt:.2f} s"}


def _config(n: int, nb: int, ws: int) -> dict:
    """The workload's config block, shared by both arms."""
    return {"workload": WORKLOAD, "batch": n, "ages": K_AGES, "metallicities": N_Z, "pixels": N_PIX,
            "filters": nb, "parallelism": f"replicas x{ws}",
            "l2": "inputs larger than L2 (673 MB of FP64 weights per step)"}


def run_reference(args) -> None:
    """The CPU implementation of the path (the FP64 oracle restating compute_csp_batch, OpenMP on every host core):
    each step is a bounded sample of --cpu-sample models of the B = --batch workload, and ms_per_step is that
    sample's measured time (the rate per model is the comparable figure)."""
    ws, rank = _dist()
    if rank != 0:
        return
    n_sample = args.cpu_sample
    vals = []
    for i in range(args.warmup + args.steps):
        r = cpu_oracle_rate(n_sample, seed=100 + i)
        if i >= args.warmup:
            vals.append(r)
    v = float(np.mean([r["value"] for r in vals]))
    ms_sample = float(np.mean([r["seconds"] for r in vals])) * 1e3
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "models/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_sample, "models_per_step": n_sample,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": _config(args.batch, 40, args.gpus),
            "note": "OpenSPS is Fortran (no Fortran compiler in this image or on the GPU host): the FP64 C oracle "
                    "restating its compute_csp_batch is the CPU implementation timed; each step is a sample of "
                    f"{n_sample} models of the workload and ms_per_step is that sample's measured time",
            "cpu_baseline": {"value": v, "unit": "models/s", "cores": vals[0]["cores"], "kind": "port",
                             "sample": vals[0]["sample"]},
            "e2e": {"value": v, "unit": "models/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def adjoint_measure(ctx, args, rank, torch, barrier) -> dict | None:
    """The reverse pass (compute_csp_batch_grad_rows) at B = --adjoint-batch through the C API from page-locked host
    buffers: weights, magnitude and spectrum cotangents (N(0, 1) on 40 magnitudes and 512 spectral bins) in;
    magnitudes, mass, L_bol, params_bar and weights_z_bar out. Wall time per call, and the device time of its
    stages (CUDA events on the library's stream)."""
    from libopensps_gb300 import workloads
    n = args.adjoint_batch
    if n <= 0:
        return None
    ns, nb = ctx.nspec, ctx.nbands
    h_wz = torch.empty((n, N_Z, K_AGES), dtype=torch.float64, pin_memory=True)
    _, params = workloads.mixed_csp(n, seed=2000 + rank, out=h_wz.numpy())
    mb, sb = workloads.adjoint_cotangents(n, ns, nb, seed=4)
    h_mb = torch.from_numpy(mb).pin_memory().numpy()
    h_sb = torch.from_numpy(sb).pin_memory().numpy()
    out = {"mags": (n, nb), "mass": (n,), "lbol": (n,), "params_bar": (n, 44), "weights_z_bar": (n, N_Z, K_AGES)}
    out = {k: torch.empty(v, dtype=torch.float64, pin_memory=True).numpy() for k, v in out.items()}
    wz = h_wz.numpy()
    steps, warm = args.adjoint_steps, max(args.warmup, 1)

    def call():
        ctx.csp_batch_grad(params, wz, mags_bar=h_mb, spec_bar=h_sb, spec=False, out=out)

    for _ in range(warm):
        call()
    barrier()
    ctx.set_profiling(True)
    t0 = time.perf_counter()
    for _ in range(steps):
        call()
    barrier()
    ms = (time.perf_counter() - t0) * 1e3 / steps
    kt = ctx.kernel_times()
    ctx.set_profiling(False)
    names = ["model_params", "weight_operand_and_fp64_sums", "contract", "bands", "-", "copies_host", "adjoint",
             "weights_gemm", "weights_cotangent"]
    stages = dict(zip(names, kt))
    dev = sum(v for k, v in stages.items() if k != "copies_host")
    h2d = wz.nbytes + h_mb.nbytes + h_sb.nbytes + n * 11 * 8
    d2h = sum(a.nbytes for a in out.values())
    return {"batch": n, "value": n / (ms * 1e-3), "unit": "models/s", "ms_per_step": ms, "steps": steps,
            "device_ms": dev, "device_value": n / (dev * 1e-3) if dev > 0 else None, "stage_ms": stages,
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "cotangents": "N(0,1) on 40 magnitudes and 512 spectral bins (FP32 values)",
            "outputs": "mags, mass, lbol, params_bar (44 rows), weights_z_bar"}


def ssp_operator_measure(args, torch, barrier) -> dict | None:
    """The SSP operator with a Kroupa IMF per model (slopes uniform in [0.3, 1.8], [1.3, 2.8], [1.8, 3.3]) at B =
    --ops-batch through the C API (weights over ages and metallicities of the mixed workload: every grid point holds
    weight, so 1284 x 1500 IMF bin weights per model), wall time per call with its device stage times."""
    from libopensps_gb300 import workloads
    from libopensps_gb300.capi import Context
    n = args.ops_batch
    if n <= 0:
        return None
    ctx = Context()
    ctx.set_int("add_igm_absorption", 1)
    ctx.build_ssp_ops()
    h_wz = torch.empty((n, N_Z, K_AGES), dtype=torch.float64, pin_memory=True)
    _, params = workloads.mixed_csp(n, seed=3000, out=h_wz.numpy())
    rng = np.random.default_rng(3001)
    params = dict(params, imf1=rng.uniform(0.3, 1.8, n), imf2=rng.uniform(1.3, 2.8, n), imf3=rng.uniform(1.8, 3.3, n))
    wz = h_wz.numpy()
    for _ in range(max(args.warmup, 1)):
        ctx.csp_batch(params, ssp_weights_z=wz, spec=False)
    barrier()
    ctx.set_profiling(True)
    t0 = time.perf_counter()
    for _ in range(args.ops_steps):
        ctx.csp_batch(params, ssp_weights_z=wz, spec=False)
    barrier()
    ms = (time.perf_counter() - t0) * 1e3 / args.ops_steps
    kt = ctx.kernel_times()
    interp = ctx.ops_last_interpolated()
    ctx.set_profiling(False)
    # the exact fold on the same batch, for comparison (a few steps)
    ctx.set_int("gb300_ops_exact", 1)
    ctx.csp_batch(params, ssp_weights_z=wz, spec=False)
    ctx.set_profiling(True)
    for _ in range(3):
        ctx.csp_batch(params, ssp_weights_z=wz, spec=False)
    kt_exact = ctx.kernel_times()
    ctx.set_profiling(False)
    ctx.close()
    names = ["model_params", "fold_and_template_gemm", "epilogue", "bands"]
    stages = dict(zip(names, kt))
    dev = sum(stages.values())
    return {"batch": n, "value": n / (ms * 1e-3), "unit": "models/s", "ms_per_step": ms, "steps": args.ops_steps,
            "fold": "interpolated (tcgen05 GEMM against the Lagrange basis in ln m)" if interp else "exact",
            "exact_fold_stage_ms": dict(zip(names, kt_exact)),
            "device_ms": dev, "device_value": n / (dev * 1e-3) if dev > 0 else None, "stage_ms": stages,
            "imf_bin_weights_per_model": K_AGES * N_Z * 1500, "operator_entries": K_AGES * N_Z * 1500 * 4,
            "workload": "IMF-free CSP through the SSP operator (Kroupa slopes per model), mixed-workload weights, "
                        "power-law dust, z 0-6 with IGM, smoothing 50-300 km/s, 40 filters"}


def ssp_operator_grad_measure(args, torch, barrier) -> dict | None:
    """The reverse pass through the SSP operator: the operator leg's batch (Kroupa slopes per model) at B =
    --ops-grad-batch with N(0,1) magnitude cotangents (FP64, page-locked), params_bar with the imf1-3 rows and the
    weights' cotangent over ages and metallicities, through compute_csp_batch_grad; wall time per call with the
    device stage times (the forward's, the adjoint, the template-cotangent GEMMs and the reverse fold)."""
    from libopensps_gb300 import workloads
    from libopensps_gb300.capi import Context
    n = args.ops_grad_batch
    if n <= 0:
        return None
    ctx = Context()
    ctx.set_int("add_igm_absorption", 1)
    ctx.build_ssp_ops()
    h_wz = torch.empty((n, N_Z, K_AGES), dtype=torch.float64, pin_memory=True)
    _, params = workloads.mixed_csp(n, seed=3100, out=h_wz.numpy())
    rng = np.random.default_rng(3101)
    params = dict(params, imf1=rng.uniform(0.3, 1.8, n), imf2=rng.uniform(1.3, 2.8, n), imf3=rng.uniform(1.8, 3.3, n))
    h_mb = torch.empty((n, ctx.nbands), dtype=torch.float64, pin_memory=True).numpy()
    h_mb[:] = rng.standard_normal(h_mb.shape)
    out = {"mags": torch.empty((n, ctx.nbands), dtype=torch.float64, pin_memory=True).numpy(),
           "mass": torch.empty(n, dtype=torch.float64, pin_memory=True).numpy(),
           "lbol": torch.empty(n, dtype=torch.float64, pin_memory=True).numpy(),
           "weights_z_bar": torch.empty((n, N_Z, K_AGES), dtype=torch.float64, pin_memory=True).numpy()}
    wz = h_wz.numpy()

    def call():
        return ctx.csp_batch_grad(params, wz, mags_bar=h_mb, spec=False, out=out)

    for _ in range(max(args.warmup, 1)):
        call()
    barrier()
    ctx.set_profiling(True)
    t0 = time.perf_counter()
    for _ in range(args.ops_grad_steps):
        r = call()
    barrier()
    ms = (time.perf_counter() - t0) * 1e3 / args.ops_grad_steps
    kt = ctx.kernel_times()
    interp = ctx.ops_last_interpolated()
    ctx.set_profiling(False)
    ctx.close()
    names = ["model_params", "fold_and_template_gemm", "epilogue", "bands", "-", "copies_host", "adjoint",
             "template_cotangent_gemm", "reverse_fold"]
    stages = dict(zip(names, kt))
    dev = sum(v for k, v in stages.items() if k != "copies_host")
    return {"batch": n, "value": n / (ms * 1e-3), "unit": "models/s", "ms_per_step": ms, "steps": args.ops_grad_steps,
            "fold": "interpolated" if interp else "exact", "device_ms": dev,
            "device_value": n / (dev * 1e-3) if dev > 0 else None, "stage_ms": stages,
            "params_bar_rows": int(r["params_bar"].shape[1]),
            "workload": "the operator leg's batch with N(0,1) cotangents on 40 magnitudes: params_bar (imf1-3 rows "
                        "included) and weights_z_bar"}


def fp64_measure(args, torch, barrier) -> dict | None:
    """The plain FP64 path of the same workload ("gb300_fp64": DGEMM age sums, every later stage in FP64) at B =
    --fp64-batch through the C API: the denominator of the mixed path's speed-up (device stage times alongside)."""
    from libopensps_gb300 import workloads
    from libopensps_gb300.capi import Context
    n = args.fp64_batch
    if n <= 0:
        return None
    ctx = Context()
    ctx.set_int("add_neb_emission", 1)
    ctx.set_int("add_igm_absorption", 1)
    ctx.set_int("gb300_fp64", 1)
    h_wz = torch.empty((n, N_Z, K_AGES), dtype=torch.float64, pin_memory=True)
    _, params = workloads.mixed_csp(n, seed=4000, out=h_wz.numpy())
    wz = h_wz.numpy()
    ctx.csp_batch(params, ssp_weights_z=wz, spec=False)
    barrier()
    ctx.set_profiling(True)
    t0 = time.perf_counter()
    for _ in range(args.fp64_steps):
        ctx.csp_batch(params, ssp_weights_z=wz, spec=False)
    barrier()
    ms = (time.perf_counter() - t0) * 1e3 / args.fp64_steps
    kt = ctx.kernel_times()
    ctx.set_profiling(False)
    ctx.close()
    dev = sum(kt[:5])
    return {"batch": n, "value": n / (ms * 1e-3), "unit": "models/s", "ms_per_step": ms, "steps": args.fp64_steps,
            "device_ms": dev, "device_value": n / (dev * 1e-3) if dev > 0 else None,
            "stage_ms": dict(zip(["model_params", "age_sums_dgemm_and_fp64_tail", "-", "-", "fp64_sums"], kt)),
            "dtype": "f64"}


def emulator_measure(args, torch, barrier) -> dict | None:
    """The learned emulator (the shipped five-member ensemble) at B = --emu-batch: inputs drawn over its training box
    (seed 77). Device-resident timing of the fused inference kernel (CUDA events on the library's stream; inputs
    42 MB, outputs 0.44 GB per step: larger than L2), the flagged fraction (ensemble spread > 0.01 mag or outside the
    box), end to end through the C API from host arrays with the flagged models computed by the plain CSP, the
    accuracy against the plain CSP on a 4096-model sample, and the plain CSP of the same physics (the SSP operator
    with the IMF per model, the delayed-tau SFH) on 65536 of the models."""
    from libopensps_gb300.capi import EMU_INPUTS
    from libopensps_gb300.emulator import WEIGHTS, training_context
    n = args.emu_batch
    if n <= 0 or not WEIGHTS.exists():
        return None
    ctx = training_context()
    ctx.emulator_load(WEIGHTS)
    ctx.emulator_set_threshold(0.01, 15.0)
    lo = np.array([0.1, 1.0, -2.0, 0.0, -1.0, 0.0, 50.0, 0.3, 1.3, 1.8])
    hi = np.array([10.0, 13.7, 0.5, 3.0, -0.4, 6.0, 300.0, 1.8, 2.8, 3.3])
    rng = np.random.default_rng(77)
    x = lo + (hi - lo) * rng.uniform(size=(n, 10))
    x[:, 0] = 10.0 ** rng.uniform(-1.0, 1.0, size=n)
    nb = ctx.nbands
    dev = torch.device("cuda")
    d_x = torch.from_numpy(x.astype(np.float32)).to(dev)
    d_mags = torch.empty((n, nb), dtype=torch.float32, device=dev)
    d_pca = torch.empty((n, 64), dtype=torch.float32, device=dev)
    d_spread = torch.empty(n, dtype=torch.float32, device=dev)
    d_flag = torch.empty(n, dtype=torch.int32, device=dev)
    d_flagged = torch.empty(n, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()

    def call(count=False):
        return ctx.emulator_predict_device(n, d_x.data_ptr(), d_mags.data_ptr(), d_flag.data_ptr(),
                                           d_flagged.data_ptr(), d_pca.data_ptr(), d_spread.data_ptr(),
                                           count=count, sync=False)

    nflag = call(count=True)
    for _ in range(max(args.warmup, 3)):
        call()
    st = torch.cuda.ExternalStream(ctx.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(args.emu_steps):
        call()
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.emu_steps
    value = n / (ms * 1e-3)
    flops = 5 * 2.0 * (512 * 32 + 3 * 512 * 512 + 128 * 512) * n
    pk = _peaks()
    # end to end from host arrays, the flagged models through the plain CSP
    ctx.emulator_predict(x[:4096], fallback=True)
    t0 = time.perf_counter()
    for _ in range(args.emu_e2e_steps):
        out = ctx.emulator_predict(x, fallback=True)
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.emu_e2e_steps
    # accuracy against the plain CSP, and the plain CSP's own rate on the same physics
    ns = 4096
    ref = ctx.csp_batch({k: x[:ns, i] for i, k in enumerate(EMU_INPUTS)}, spec=False)["mags"]
    emu = ctx.emulator_predict(x[:ns], fallback=False)
    mmin = np.min(np.where(np.isfinite(ref), ref, np.inf), axis=1, keepdims=True)
    gate = np.isfinite(ref) & (ref < mmin + 15.0)
    err = np.where(gate, np.abs(emu["mags"] - ref), 0.0).max(axis=1)
    ok = emu["source"] == 0
    nc = min(n, 65536)
    params = {k: x[:nc, i] for i, k in enumerate(EMU_INPUTS)}
    ctx.csp_batch({k: v[:1024] for k, v in params.items()}, spec=False)
    t0 = time.perf_counter()
    ctx.csp_batch(params, spec=False)
    csp_rate = nc / (time.perf_counter() - t0)
    ctx.close()
    return {"batch": n, "value": value, "unit": "models/s", "ms_per_step": ms, "steps": args.emu_steps,
            "dtype": "f16 weights and activations (inputs split hi + lo), f32 accumulate",
            "roofline": {"bound": "tensor", "achieved": flops / (ms * 1e-3) / 1e12, "peak": pk["bf16_tflops_sustained"],
                         "unit": "TFLOP/s", "frac": flops / (ms * 1e-3) / 1e12 / pk["bf16_tflops_sustained"],
                         "kernel": "emu_infer_kernel", "flop_per_model": flops / n,
                         "peak_src": f"{pk['src']} sustained dense bf16 (f16 runs at the same rate)"},
            "flagged_frac": nflag / n,
            "e2e": {"value": n / (e2e_ms * 1e-3), "unit": "models/s", "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": int(n * 10 * 4), "d2h_bytes_per_step": int(n * (nb + 1) * 4 + n * 4),
                    "fallback_models": int(out["n_fallback"]),
                    "outputs": "mags (flagged models from the plain CSP)"},
            "accuracy_vs_csp": {"sample": ns, "unflagged_within_0.01_mag": float(np.mean(err[ok] <= 0.01)),
                                "unflagged_max_mag": float(err[ok].max()), "all_p99_mag": float(np.percentile(err, 99)),
                                "flagged_frac": float(1 - ok.mean()),
                                "bands": "less than 15 mag fainter than the model's brightest"},
            "csp_same_physics": {"batch": nc, "value": csp_rate, "unit": "models/s",
                                 "workload": "SSP operator with the Kroupa slopes per model, delayed-tau SFH on the "
                                             "device, dust, z 0-6 with IGM, smoothing, 40 filters (end to end)"},
            "speedup_vs_same_physics_csp": value / csp_rate, "e2e_speedup_vs_same_physics_csp": (n / (e2e_ms * 1e-3)) / csp_rate}


def sfh_config_measure(args, torch, barrier) -> dict | None:
    """The plain batched CSP of the delayed-tau configuration at B = --sfh-batch (256): tau log-uniform 0.1-10 Gyr,
    tage uniform 1-13.7 Gyr, logZ uniform -2..0.5 (the two-slab blend), power-law dust tau_V uniform 0-2 with slope
    -0.7, z = 0, no nebular emission, 20 Gaussian filters; spectra (FP64) and magnitudes to the host. Timed through the
    C API on the mixed path and on the plain FP64 GPU path (SFH weights formed on the device in both), and the FP64 CPU
    oracle (OpenMP, the machine's cores) on the same models."""
    from libopensps_gb300 import synthdata
    from libopensps_gb300.capi import Context
    from oracle.oracle import Oracle, SFH_NAMES, blend_at_logzsol, sfh_weights
    n = args.sfh_batch
    if n <= 0:
        return None
    rng = np.random.default_rng(0)
    params = {"tau": 10.0 ** rng.uniform(-1.0, 1.0, n), "tage": rng.uniform(1.0, 13.7, n),
              "logzsol": rng.uniform(-2.0, 0.5, n), "dust2": rng.uniform(0.0, 2.0, n), "dust_index": np.full(n, -0.7)}
    out = {}
    for name, fp64 in (("mixed", 0), ("fp64", 1)):
        ctx = Context()
        ctx.set_filters_library("gauss20")
        ctx.set_int("sfh", 4)
        ctx.set_int("gb300_fp64", fp64)
        try:
            for _ in range(max(args.warmup, 1)):
                ctx.csp_batch(params)
            t0 = time.perf_counter()
            for _ in range(args.sfh_steps):
                ctx.csp_batch(params)
            out[name] = n / ((time.perf_counter() - t0) / args.sfh_steps)
        except Exception as exc:          # a path that refuses the configuration: reported, not fatal
            out[name] = f"unavailable: {exc}"
        ctx.close()
    data = synthdata.load()
    o = Oracle(data, nbands=20, add_neb=False, add_igm=False)
    t0 = time.perf_counter()
    w, _ = sfh_weights(data["log_age"], 4, params, n)
    wz, _ = blend_at_logzsol(data, w, params["logzsol"])
    o.csp_batch({k: v for k, v in params.items() if k not in SFH_NAMES and k != "logzsol"}, wz)
    cpu = n / (time.perf_counter() - t0)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"batch": n, "unit": "models/s", "mixed_e2e": out["mixed"], "fp64_gpu_e2e": out["fp64"],
            "cpu_oracle": {"value": cpu, "cores": cores, "kind": "port"},
            "outputs": "spectra (FP64) and 20 magnitudes to the host",
            "workload": "delayed-tau SFH on the device, logZ blend, power-law dust, z = 0, no nebular emission"}


def dust_emission_measure(ctx, params, h_wz, args, barrier) -> dict | None:
    """The headline batch (B = --batch, nebular lines, IGM) with dust emission (the Draine & Li energy balance) and
    the AGN torus switched on: per-model q_PAH, U_min, gamma, fagn and tau_AGN, and the birth-cloud, diffuse and
    extra screens that set what is absorbed. Timed end to end through the C API from the same pinned host weights as
    the headline e2e (magnitudes, mass and L_bol back to the host)."""
    from libopensps_gb300 import synth_dust
    n = h_wz.shape[0]
    if args.dust_steps <= 0:
        return None
    synth_dust.generate()
    synth_dust.generate_agn()
    rng = np.random.default_rng(77)
    # (frac_obrun stays 0 as in the headline batch; the escaping ionizing light above 0 has its own leg)
    p = dict(params, dust1=rng.uniform(0.1, 1.0, n), dust3=rng.uniform(0.0, 0.4, n),
             duste_qpah=rng.uniform(0.5, 4.5, n),
             duste_umin=rng.uniform(0.1, 25.0, n), duste_gamma=rng.uniform(0.0, 0.5, n),
             fagn=rng.uniform(0.0, 1.0, n), agn_tau=rng.uniform(5.0, 150.0, n))
    ctx.set_int("add_dust_emission", 1)
    ctx.set_int("add_agn_dust", 1)
    try:
        for i in range(args.warmup + args.dust_steps):
            if i == args.warmup:
                barrier()
                t0 = time.perf_counter()
            ctx.csp_batch(p, ssp_weights_z=h_wz, spec=False)
        barrier()
        ms = (time.perf_counter() - t0) * 1e3 / args.dust_steps
    finally:
        ctx.set_int("add_dust_emission", 0)
        ctx.set_int("add_agn_dust", 0)
    return {"batch": n, "unit": "models/s", "e2e": n / (ms * 1e-3), "ms_per_step": ms,
            "workload": "headline batch + dust emission (7 q_PAH x 22 U_min templates) + AGN torus (9 tau)"}


def escaping_light_measure(ctx, params, h_wz, args, barrier, torch) -> dict | None:
    """The headline batch with frac_obrun uniform in 0-0.5: the nebular ages' escaping ionizing light (nebular
    emission's gas absorption with an escaping fraction per model) as extra K blocks of the contraction on the pixel
    tiles below 912 A. Timed end to end through the C API from the same pinned host weights as the headline e2e, and
    device-resident (opensps_gb300_batch_device, CUDA events on the library's stream)."""
    from libopensps_gb300 import workloads
    n = h_wz.shape[0]
    if args.ion_steps <= 0:
        return None
    rng = np.random.default_rng(78)
    p = dict(params, frac_obrun=rng.uniform(0.0, 0.5, n))
    for i in range(args.warmup + args.ion_steps):
        if i == args.warmup:
            barrier()
            t0 = time.perf_counter()
        ctx.csp_batch(p, ssp_weights_z=h_wz, spec=False)
    barrier()
    ms = (time.perf_counter() - t0) * 1e3 / args.ion_steps
    d_wz = torch.from_numpy(h_wz).to("cuda")
    d_par = torch.from_numpy(workloads.device_param_table(p, n)).to("cuda")
    d_mags = torch.empty((n, ctx.nbands), dtype=torch.float64, device="cuda")
    stream = torch.cuda.ExternalStream(ctx.stream())
    for _ in range(args.warmup):
        ctx.batch_device(n, d_par.data_ptr(), d_wz.data_ptr(), d_mags.data_ptr(), sync=False)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.ion_steps):
        ctx.batch_device(n, d_par.data_ptr(), d_wz.data_ptr(), d_mags.data_ptr(), sync=False)
    e1.record(stream)
    barrier()
    dms = e0.elapsed_time(e1) / args.ion_steps
    del d_wz, d_par, d_mags
    return {"batch": n, "unit": "models/s", "e2e": n / (ms * 1e-3), "ms_per_step": ms,
            "device_value": n / (dms * 1e-3), "device_ms": dms,
            "workload": "headline batch with frac_obrun uniform 0-0.5 (the nebular ages' escaping ionizing light: 420 "
                        "more K columns of the contraction on the 17 pixel tiles below 912 A)"}


def nebular_continuum_measure(params, h_wz, args, barrier) -> dict | None:
    """The headline batch with the CLOUDY-grid nebular continuum: a standard-format data root holding the synthetic
    libraries and a CLOUDY-style grid (nebular/synthetic_nodust, 11 log Z x 10 ages x 7 log U), gas_logz and gas_logu
    per model, frac_obrun uniform 0-0.4. The continuum joins the young and old sums in the per-model epilogue (the
    batch's parts path, in 16384-model chunks). Timed end to end through the C API from the same pinned host weights
    as the headline e2e."""
    import shutil
    from libopensps_gb300 import stdformat, synthdata
    from libopensps_gb300.capi import Context
    n = h_wz.shape[0]
    if args.neb_steps <= 0:
        return None
    root = Path(tempfile.mkdtemp(prefix="opensps_neb_"))
    old = os.environ.get("OPENSPS_DATA_HOME")
    try:
        stdformat.convert_synthetic(root, src_root=synthdata.default_root(), dust=False, agn=False, nebular=True)
        c = Context(data_root=root)
        c.set_int("add_neb_emission", 1)
        c.set_int("add_igm_absorption", 1)
        rng = np.random.default_rng(79)
        p = dict(params, gas_logz=rng.uniform(-2.0, 0.2, n), gas_logu=rng.uniform(-4.0, -1.0, n),
                 frac_obrun=rng.uniform(0.0, 0.4, n))
        for i in range(args.warmup + args.neb_steps):
            if i == args.warmup:
                barrier()
                t0 = time.perf_counter()
            c.csp_batch(p, ssp_weights_z=h_wz, spec=False)
        barrier()
        ms = (time.perf_counter() - t0) * 1e3 / args.neb_steps
        c.close()
    finally:
        if old is not None:
            os.environ["OPENSPS_DATA_HOME"] = old
        shutil.rmtree(root, ignore_errors=True)
    return {"batch": n, "unit": "models/s", "e2e": n / (ms * 1e-3), "ms_per_step": ms,
            "workload": "headline batch + CLOUDY-grid nebular continuum (gas_logz, gas_logu, frac_obrun per model)"}


def run_ours(args) -> None:
    import torch
    ws, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from libopensps_gb300 import workloads
    from libopensps_gb300.capi import Context

    n = args.batch
    ctx = Context()
    ctx.set_int("add_neb_emission", 1)
    ctx.set_int("add_igm_absorption", 1)
    nb = ctx.nbands

    # inputs: pinned host copies (for e2e) and device-resident copies (for value)
    h_wz = torch.empty((n, N_Z, K_AGES), dtype=torch.float64, pin_memory=True)
    _, params = workloads.mixed_csp(n, seed=1000 + rank, out=h_wz.numpy())
    h_par = torch.from_numpy(workloads.device_param_table(params, n)).pin_memory()
    d_wz = h_wz.to("cuda", non_blocking=False)
    d_par = h_par.to("cuda", non_blocking=False)
    d_mags = torch.empty((n, nb), dtype=torch.float64, device="cuda")
    stream = torch.cuda.ExternalStream(ctx.stream())

    def step():
        ctx.batch_device(n, d_par.data_ptr(), d_wz.data_ptr(), d_mags.data_ptr(), sync=False)

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        step()
    barrier()
    clocks = ClockSampler(Path(tempfile.gettempdir()) / f"opensps_clocks_{os.getpid()}_{rank}.csv")
    clocks.start()
    time.sleep(0.3)
    ctx.set_profiling(True)
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    barrier()
    ms = ev0.elapsed_time(ev1)
    ktimes = ctx.kernel_times()
    ctx.set_profiling(False)
    launches = ctx.last_launches()
    clk = clocks.stop()
    if ws > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    value = ws * n / (ms_step * 1e-3)

    # e2e through the C API from pinned host buffers (magnitudes, mass and L_bol back to the host)
    e2e_ms = None
    h_wz_np = h_wz.numpy()
    for i in range(args.warmup + args.steps):
        if i == args.warmup:
            barrier()
            t0 = time.perf_counter()
        ctx.csp_batch(params, ssp_weights_z=h_wz_np, spec=False)
    barrier()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    if ws > 1:
        t = torch.tensor([e2e_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(t.item())
    h2d = h_wz.numel() * 8 + n * 11 * 8 + 3 * n * 8
    d2h = n * nb * 8 + 6 * n * 8
    # the same from pageable host weights (an ordinary numpy array, as a Fortran or Python caller hands them): read in
    # place by the operand kernel where the device reads pageable memory
    h_wz_pageable = np.array(h_wz_np)
    for i in range(args.warmup + args.steps):
        if i == args.warmup:
            barrier()
            t0 = time.perf_counter()
        ctx.csp_batch(params, ssp_weights_z=h_wz_pageable, spec=False)
    barrier()
    e2e_pageable_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    in_place = ctx.last_input_in_place()
    del h_wz_pageable
    dust_em = dust_emission_measure(ctx, params, h_wz_np, args, barrier)
    esc = escaping_light_measure(ctx, params, h_wz_np, args, barrier, torch)
    neb_cont = nebular_continuum_measure(params, h_wz_np, args, barrier)
    adjoint = adjoint_measure(ctx, args, rank, torch, barrier)
    ssp_ops = ssp_operator_measure(args, torch, barrier)
    ssp_ops_grad = ssp_operator_grad_measure(args, torch, barrier)
    fp64 = fp64_measure(args, torch, barrier)
    sfh_cfg = sfh_config_measure(args, torch, barrier) if rank == 0 else None
    emulator = emulator_measure(args, torch, barrier) if rank == 0 else None
    if emulator:
        emulator["speedup_vs_mixed_csp"] = emulator["value"] / value

    # roofline of the contraction
    pk = _peaks()
    flops = 3.0 * 2.0 * (K_AGES * N_Z) * N_PIX * n
    t_contract = ktimes[2] if len(ktimes) > 2 else None
    achieved = flops / (t_contract * 1e-3) / 1e12 if t_contract else None
    traffic = None
    prof = ROOT / "profiles" / "traffic.json"
    if prof.exists():
        traffic = json.loads(prof.read_text()).get("csp_contract_kernel_bytes_per_launch_at_65536")

    if rank == 0:
        cpu = cpu_oracle_rate(args.cpu_sample) if args.cpu_sample > 0 else None
        line = {
            "metric": METRIC, "value": value, "unit": "models/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16x3 (split-BF16, f32 accumulate; FP64 sums)", "data": "synthetic",
            "config": _config(n, nb, ws),
            "e2e": {"value": ws * n / (e2e_ms * 1e-3), "unit": "models/s",
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "outputs": "mags, mass, lbol (spectra stay on the device)"},
            "e2e_pageable": {"value": ws * n / (e2e_pageable_ms * 1e-3), "unit": "models/s",
                             "weights": "pageable host memory", "read_in_place": in_place},
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": pk["bf16_tflops_sustained"],
                         "unit": "TFLOP/s", "frac": (achieved / pk["bf16_tflops_sustained"]) if achieved else None,
                         "traffic": traffic, "kernel": "csp_contract_kernel<1>",
                         "peak_src": f"{pk['src']} sustained bf16",
                         "stage_ms": dict(zip(["model_params", "weight_operand_and_fp64_sums", "contract", "bands"],
                                              ktimes))},
            "cpu_baseline": cpu,
            "adjoint": adjoint,
            "ssp_operator": ssp_ops,
            "ssp_operator_grad": ssp_ops_grad,
            "fp64_path": fp64,
            "mixed_over_fp64": (value / fp64["device_value"]) if fp64 and fp64.get("device_value") else None,
            "sfh_config": sfh_cfg,
            "emulator": emulator,
            "dust_emission": dict(dust_em, over_plain_e2e=dust_em["e2e"] / (n / (e2e_ms * 1e-3))) if dust_em else None,
            "nebular_continuum": dict(neb_cont, e2e_ms_over_plain=neb_cont["ms_per_step"] / e2e_ms) if neb_cont else None,
            "escaping_light": dict(esc, e2e_ms_over_plain=esc["ms_per_step"] / e2e_ms,
                                   device_ms_over_plain=esc["device_ms"] / ms_step) if esc else None,
            "gpu_launches": launches * args.steps,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--cpu-sample", type=int, default=4096)
    ap.add_argument("--adjoint-batch", type=int, default=16384)
    ap.add_argument("--adjoint-steps", type=int, default=10)
    ap.add_argument("--ops-batch", type=int, default=1024)
    ap.add_argument("--ops-steps", type=int, default=10)
    ap.add_argument("--ops-grad-batch", type=int, default=1024)
    ap.add_argument("--ops-grad-steps", type=int, default=5)
    ap.add_argument("--fp64-batch", type=int, default=65536)
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--sfh-batch", type=int, default=256)
    ap.add_argument("--sfh-steps", type=int, default=20)
    ap.add_argument("--emu-batch", type=int, default=1048576)
    ap.add_argument("--emu-steps", type=int, default=20)
    ap.add_argument("--emu-e2e-steps", type=int, default=2)
    ap.add_argument("--dust-steps", type=int, default=10)
    ap.add_argument("--ion-steps", type=int, default=10)
    ap.add_argument("--neb-steps", type=int, default=5)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
