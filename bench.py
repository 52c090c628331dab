"""Benchmark: baryon two-point contractions on a 24^3 x 64 lattice (one GB300).

Workload ("baryon_2pt_24c64"): three propagators u, u, d in PyQUDA even/odd
layout [2, 64, 24, 24, 12, 4, 4, 3, 3] -- seeded unit-variance complex Gaussian
entries times exp(-m|t|) (m = 0.25, 0.25, 0.30; the two u propagators hold the
same values in separate buffers, d has its own seed).  One step evaluates all
six contract_enum.h contraction types with Gamma_ij = Gamma_kl = C g5
(Gamma(5)) for the two projectors (1 +- g4)/2 at zero momentum, i.e. 12
site-contractions per site, reduced per timeslice.  The headline passes the
two u buffers, so it evaluates both triangle passes; ``mixed_same_field``
times the same step with one u buffer passed twice, where the library
evaluates one triangle pass (reported beside the headline, not as it).

Metric: GSite/s = site-contractions per second / 1e9 for the mixed form
(complex64 storage, FP32 arithmetic, FP64 per-timeslice reduction) with the
propagators resident in HBM; the plain complex128 form, per-call and fused, is
measured beside it, and the per-timeslice relative error of the mixed form
against the plain FP64 form is reported.  ``e2e`` repeats the measurement
through the C ABI from pinned host complex128 buffers
(contract_baryon_all_types_host: timeslice chunks copied back to back on one copy stream,
converted to complex64 and contracted as they arrive), with every
host->device copy, the conversion and the read-back of the correlators inside
the timed region.

``--impl reference`` times the reference's CPU arithmetic for the same
workload on the host cores (see ``oracle/``).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

LATT = (24, 24, 24, 64)
MASSES = (0.25, 0.25, 0.30)
GAMMA_CG5 = 5
N_TYPES = 6
N_PROJ = 2
UNITS_PER_SITE = N_TYPES * N_PROJ
# Complex FMAs per site of the fused kernel's shared-wedge form (16 threads per site, one
# (i, x) pair each): 4 wedges a ^ P_j[j][n] (36 each), each dotted with the N blocks of
# both triangle passes for the 2 gamma-basis terms (4 x 9), the loop form's 2 x 9 dots
# with Q_w, and the projector coefficients 2 x 2 x 2; Q set-up 18 x 3.  8 flops per
# complex FMA.
FUSED_CFMA_PER_SITE = 16 * (4 * (36 + 4 * 9) + 2 * 9 + 2 * 2 * 2) + 18 * 3
# The compiled op behind each tile-shape name of the fused complex64 pass.
FUSED_KERNELS = {"shared": "BaryonFusedSharedWedgeOp", "merged": "BaryonFusedCliffMergedOp",
                 "shared_same": "BaryonFusedSharedWedgeSameOp", "same": "BaryonFusedCliffMergedOp (SAMEIJ)",
                 "cw": "BaryonFusedCliffOp"}
WORKLOAD = "baryon_2pt_24c64"
METRIC = "GSite/s & HBM GB/s: mixed vs FP64 GPU contraction at <=1e-6 rel err/timeslice"


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """Per-launch DRAM bytes of the fused kernel from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "baryon_fused_c64_24c64.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "gloo" if args.impl == "reference" else "nccl"
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world, device=None):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank, ms_max, world):
    """Whole-job GSite/s of `world` independent replicas: every rank processes
    `units_per_rank` site-contractions and the job takes the slowest rank's time."""
    return world * units_per_rank / (ms_max * 1e-3) / 1e9


# ------------------------------------------------------------ CPU baseline --

def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return None


def sample_slices(prop, n):
    """The first `n` timeslices of a device propagator [V, 4, 4, 3, 3] (PyQUDA
    even/odd order) as a host complex128 array -- itself the even/odd layout of
    the (Lx, Ly, Lz, n) sub-lattice."""
    lx, ly, lz, lt = LATT
    half = lx * ly * lz // 2
    sub = prop.reshape(2, lt, half, 144)[:, :n].contiguous()
    return sub.cpu().numpy().astype(np.complex128).reshape(-1, 4, 4, 3, 3)


def benchmark_inputs(n_slices, rank=0):
    """Host copies of the first `n_slices` timeslices of the benchmark's u and d:
    the same values the GPU arm contracts (the device generator, when a GPU is
    present), else the same distribution from the host generator."""
    import torch

    from contract_gb300.lattice import synthetic_propagator
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    u = synthetic_propagator(LATT, 1000 + rank, MASSES[0], device=dev)
    d = synthetic_propagator(LATT, 3000 + rank, MASSES[2], device=dev)
    out = sample_slices(u, n_slices), sample_slices(d, n_slices)
    same = dev == "cuda"
    del u, d
    return out, same


def cpu_reference(steps, warmup, pu, pd):
    """The reference's CPU arithmetic on a bounded sample: all six types x both
    projectors over the sites of `pu`, `pu`, `pd` (a few timeslices of the
    benchmark lattice).  Returns the timing record and the per-site values."""
    from oracle import einsum_oracle as eo
    from oracle import lib as L
    L.build()
    impl, kind = L.ref_oracle(), "reference"
    if impl is None:
        impl, kind = L.c_oracle(), "port"
    g4 = eo.GAMMA[8]
    projs = [((np.eye(4) + g4) / 2).reshape(16), ((np.eye(4) - g4) / 2).reshape(16)]
    v = pu.shape[0]
    values = {}

    def step():
        for t in range(N_TYPES):
            for w, p in enumerate(projs):
                values[t, w] = impl.baryon_general_two_point(pu, pu, pd, t, GAMMA_CG5, GAMMA_CG5, p)

    for _ in range(warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(max(1, steps)):
        step()
    dt = (time.perf_counter() - t0) / max(1, steps)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    slices = v // (LATT[0] * LATT[1] * LATT[2])
    rec = {"value": v * UNITS_PER_SITE / dt / 1e9, "unit": "GSite/s", "cores": cores, "cpu_model": cpu_model(),
           "kind": kind,
           "sample": f"{slices} of {LATT[3]} timeslices ({v} sites) x 6 types x 2 projectors, FP64, OpenMP",
           "seconds_per_step": dt}
    site = np.stack([np.stack([values[t, w] for w in range(N_PROJ)]) for t in range(N_TYPES)])
    return rec, site


def accuracy_vs_oracle(got, site, n_slices, tol_strict):
    """Per-timeslice error of GPU results `got` [6, 2, >= n] against the oracle's
    per-site values `site` [6, 2, V_sample]: strict |d_t| / |C_t| and the
    sigma-normalised |d_t| / max(|C_t|, sigma_t), each with its pass/fail."""
    from oracle import einsum_oracle as eo
    sub = LATT[:3] + (n_slices,)
    ref = eo.timeslice_sum(site, sub)
    sig = np.sqrt(eo.timeslice_sum(np.abs(site) ** 2, sub).real)
    d = np.abs(np.asarray(got)[..., :n_slices] - ref)
    strict = d / np.abs(ref)
    norm = d / np.maximum(np.abs(ref), sig)
    return {"timeslices": n_slices, "max_rel_err_strict": float(strict.max()),
            "frac_le_tol_strict": float((strict <= tol_strict).mean()), "pass_strict": bool(strict.max() <= tol_strict),
            "max_rel_err_sigma_normalised": float(norm.max()), "pass_sigma_normalised": bool(norm.max() <= tol_strict),
            "tolerance": tol_strict}


def reference_gpu_leg(args):
    """The reference's own CUDA kernels (its translation units compiled unmodified
    to sm_103a cubins, launched through the driver API as its host code launches
    them) on the benchmark's twelve complex128 baryon_general_two_point calls.
    Runs in a child process; a reported baseline beside plain_c128.per_call_ms."""
    if args.no_ref_gpu:
        return None
    if not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "gpu", "baryon_general.cubin")):
        return {"unavailable": "reference cubins not built (make -C oracle refgpu)"}
    cmd = [sys.executable, "-m", "oracle.ref_gpu", "--lattice", ",".join(map(str, LATT)), "--steps", "2",
           "--warmup", "1"]
    try:
        r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    except subprocess.TimeoutExpired:
        return {"unavailable": "reference GPU leg timed out"}
    if r.returncode != 0:
        return {"unavailable": "reference GPU leg failed: " + (r.stderr.strip().splitlines() or ["?"])[-1]}
    return json.loads(r.stdout.strip().splitlines()[-1])


def workload_config(world):
    """The `config` both arms print: what is contracted, not how."""
    return {"workload": WORKLOAD, "lattice": list(LATT), "propagators": "u, u, d (u twice in separate buffers)",
            "masses": list(MASSES), "gamma_ij": "C g5 = Gamma(5)", "gamma_kl": "C g5 = Gamma(5)",
            "projectors": "(1+g4)/2, (1-g4)/2", "types": 6,
            "site_contractions_per_step": LATT[0] * LATT[1] * LATT[2] * LATT[3] * UNITS_PER_SITE,
            "l2": "inputs 3.06 GB (c64) / 6.1 GB (c128) > L2 129 MB, no flush",
            "parallelism": f"replicas x{world}"}


def fused_kernel_name(lib, v):
    """The op and tile shape the fused complex64 pass ran with at volume v (the
    tuner's choice, else the default shape)."""
    for key, name, _ in autotune_report(lib):
        if key.startswith("kind=3,prec=1,aux=2,") and f"volume={v}," in key:
            return f"{FUSED_KERNELS.get(name.split('.')[0], '?')} ({name})"
    return "BaryonFusedSharedWedgeOp (shared.cw4.tps16.st2.occ3)"


def run_reference(args, world, rank):
    if rank != 0:
        return
    (pu, pd), same = benchmark_inputs(args.cpu_slices)
    cb, _ = cpu_reference(args.steps, args.warmup, pu, pd)
    line = {
        "impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "GSite/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": cb["seconds_per_step"] * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(world),
        "cpu_baseline": dict({k: cb[k] for k in ("value", "unit", "cores", "cpu_model", "kind", "sample")},
                             inputs="the GPU arm's u, d values" if same else "host-generated, same distribution"),
        "e2e": {"value": cb["value"], "unit": "GSite/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- GPU arm --

def run_ours(args, world, rank, local):
    import torch

    from contract_gb300 import api, build
    from contract_gb300 import _lib
    from contract_gb300.lattice import synthetic_propagator

    torch.cuda.set_device(local)
    build.build()
    lib = _lib.lib()
    lib.contract_set_error_mode(1)
    lib.contract_set_autotune(0 if args.no_autotune else 1)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    lib.contract_set_stream(stream.cuda_stream)

    lx, ly, lz, lt = LATT
    v = lx * ly * lz * lt
    units = v * UNITS_PER_SITE
    latt_c = (ctypes.c_int * 4)(*LATT)
    projs = np.ascontiguousarray(api.projector_plus_minus())
    proj_ptr = projs.ctypes.data

    # resident inputs (complex128 drop-in format) and the mixed-form copies
    u = synthetic_propagator(LATT, 1000 + rank, MASSES[0], device=dev)
    u2 = u.clone()
    d = synthetic_propagator(LATT, 3000 + rank, MASSES[2], device=dev)
    u64, u264, d64 = api.to_c64(u), api.to_c64(u2), api.to_c64(d)
    out64 = torch.empty((N_TYPES, N_PROJ, lt), dtype=torch.complex128, device=dev)
    out128 = torch.empty_like(out64)
    lib.contract_workspace_reserve(lib.contract_workspace_bytes(latt_c, UNITS_PER_SITE))

    def fused(out, a, b, c, prec):
        lib.contract_baryon_all_types(out.data_ptr(), a.data_ptr(), b.data_ptr(), c.data_ptr(), v, GAMMA_CG5,
                                      GAMMA_CG5, N_PROJ, proj_ptr, prec, latt_c)

    def check():
        if lib.contract_last_error():
            raise RuntimeError(lib.contract_last_error_message().decode())

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        check()
        torch.cuda.synchronize(dev)
        barrier(world)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        e1.synchronize()
        torch.cuda.synchronize(dev)
        barrier(world)
        check()
        return e0.elapsed_time(e1) / steps  # ms

    def timed_each(fn, steps, warmup):
        """timed() with an event between steps: (mean ms, [ms of each step])."""
        for _ in range(warmup):
            fn()
        check()
        torch.cuda.synchronize(dev)
        barrier(world)
        torch.cuda.synchronize(dev)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        ev[0].record(stream)
        for k in range(steps):
            fn()
            ev[k + 1].record(stream)
        ev[-1].synchronize()
        torch.cuda.synchronize(dev)
        barrier(world)
        check()
        each = [ev[k].elapsed_time(ev[k + 1]) for k in range(steps)]
        return ev[0].elapsed_time(ev[-1]) / steps, each

    # ---- headline: mixed fused, inputs resident (3 x 1.02 GB > L2, no flush needed)
    with ClockSampler(local) as clocks:
        ms_mixed = timed(lambda: fused(out64, u64, u264, d64, 1), args.steps, args.warmup)
    ms_mixed = max_over_ranks(ms_mixed, world, dev)
    value = replica_value(units, ms_mixed, world)

    # ---- plain complex128 forms: fused, and the drop-in per-call sequence
    plain_steps = max(1, min(args.steps, 5))
    ms_plain_fused = timed(lambda: fused(out128, u, u2, d, 0), plain_steps, 1)
    corr_t = torch.empty(lt, dtype=torch.complex128, device=dev)

    def per_call():
        for t in range(N_TYPES):
            for w in range(N_PROJ):
                lib.contract_baryon(corr_t.data_ptr(), u.data_ptr(), u2.data_ptr(), d.data_ptr(), t, v, GAMMA_CG5,
                                    GAMMA_CG5, 0, projs[w].ctypes.data, 0, latt_c)

    ms_plain_call = timed(per_call, max(1, min(args.steps, 2)), 1)
    per_call_mixed = lambda: [lib.contract_baryon(corr_t.data_ptr(), u64.data_ptr(), u264.data_ptr(),  # noqa: E731
                                                  d64.data_ptr(), t, v, GAMMA_CG5, GAMMA_CG5, 0,
                                                  projs[w].ctypes.data, 1, latt_c)
                              for t in range(N_TYPES) for w in range(N_PROJ)]
    ms_mixed_call = timed(per_call_mixed, max(1, min(args.steps, 5)), 1)
    # one u buffer for P_i and P_j: the one-pass form of the fused kernel
    out_same = torch.empty_like(out64)
    ms_same = timed(lambda: fused(out_same, u64, u64, d64, 1), max(1, min(args.steps, 50)), 3)

    # ---- accuracy of the mixed form per timeslice against the plain FP64 form
    # over the whole lattice (the tests pin the FP64 form to the oracle and to
    # the reference's own GPU kernels): strict |d_t| / |C_t| and the
    # sigma-normalised |d_t| / max(|C_t|, sigma_t), sigma_t the spread of the
    # site values, which conditions C_t on these zero-mean inputs
    fused(out64, u64, u264, d64, 1)
    fused(out128, u, u2, d, 0)
    site128 = torch.empty((N_TYPES, N_PROJ, v), dtype=torch.complex128, device=dev)
    lib.contract_baryon_all_types(site128.data_ptr(), u.data_ptr(), u2.data_ptr(), d.data_ptr(), v, GAMMA_CG5,
                                  GAMMA_CG5, N_PROJ, proj_ptr, 0, None)
    sigma = (site128.abs() ** 2).reshape(N_TYPES, N_PROJ, 2, lt, -1).sum(dim=(2, 4)).sqrt().cpu().numpy()
    del site128
    # FP64 contraction of the complex64-rounded inputs: the share of the error
    # that storage rounding alone causes
    out_rnd = torch.empty_like(out128)
    fused(out_rnd, *[api.to_c128(x) for x in (u64, u264, d64)], 0)
    torch.cuda.synchronize(dev)
    a, b, r = out64.cpu().numpy(), out128.cpu().numpy(), out_rnd.cpu().numpy()
    rel = np.abs(a - b) / np.abs(b)
    norm = np.abs(a - b) / np.maximum(np.abs(b), sigma)
    same_out = out_same.cpu().numpy()
    same_diff = float(np.abs(same_out - a).max() / np.abs(a).max())
    rel_in = np.abs(r - b) / np.abs(b)
    acc = {"vs": "plain FP64 GPU form, all 64 timeslices",
           "max_rel_err_strict": float(rel.max()), "median_rel_err_strict": float(np.median(rel)),
           "frac_le_1e-6_strict": float((rel <= 1e-6).mean()), "pass_strict_1e-6": bool(rel.max() <= 1e-6),
           "max_rel_err_sigma_normalised": float(norm.max()),
           "pass_sigma_normalised_1e-6": bool(norm.max() <= 1e-6),
           "max_rel_err_strict_by_type": [float(rel[t].max()) for t in range(N_TYPES)],
           "input_rounding_only": {"max_rel_err_strict": float(rel_in.max()),
                                   "median_rel_err_strict": float(np.median(rel_in))},
           "note": ("zero-mean i.i.d. inputs: every C_t is a random walk of site values, so the strict "
                    "bound fails where C_t nears zero; accuracy_signal holds the strict bound")}

    # ---- signal-carrying inputs: u, u, d each with a coherent part shared by
    # every site (the part a wall source gives a propagator) plus site noise, so
    # that |C_t| >> sigma_t and the strict bound is well conditioned
    from contract_gb300.lattice import coherent_propagator, shifted_triple
    cu = coherent_propagator(LATT, 1000 + rank, MASSES[0], coherent_seed=7, device=dev)
    sig_dev = (cu, cu.clone(), coherent_propagator(LATT, 3000 + rank, MASSES[2], coherent_seed=8, device=dev))
    del cu
    sig64 = [api.to_c64(x) for x in sig_dev]
    sig_out64, sig_out128 = torch.empty_like(out64), torch.empty_like(out128)
    fused(sig_out64, *sig64, 1)
    fused(sig_out128, *sig_dev, 0)
    torch.cuda.synchronize(dev)
    sa, sb = sig_out64.cpu().numpy(), sig_out128.cpu().numpy()
    srel = np.abs(sa - sb) / np.abs(sb)
    acc_signal = {"vs": "plain FP64 GPU form, all 64 timeslices",
                  "inputs": ("u, u, d with u = exp(-0.25|t|) (W_u + G_u(x)), d = exp(-0.30|t|) (W_d + G_d(x)), "
                             "W one seeded spin-colour matrix per propagator"),
                  "max_rel_err_strict": float(srel.max()), "median_rel_err_strict": float(np.median(srel)),
                  "frac_le_1e-6_strict": float((srel <= 1e-6).mean()), "pass_strict_1e-6": bool(srel.max() <= 1e-6)}
    sig_host = None
    if rank == 0 and not args.no_cpu:
        sig_host = [sample_slices(x, args.cpu_slices) for x in sig_dev]
    del sig_dev, sig64
    # the reference example's inputs (one propagator shifted by -1 / 0 / +1):
    # at large t the decaying part of P +- 1 falls below complex64 resolution,
    # which the FP64 contraction of the complex64-rounded inputs shows
    pc = coherent_propagator(LATT, 1000 + rank, MASSES[0], coherent_seed=7, device=dev)
    sh = shifted_triple(pc)
    del pc
    sh64 = [api.to_c64(x) for x in sh]
    sh_out64, sh_out128, sh_rnd = torch.empty_like(out64), torch.empty_like(out128), torch.empty_like(out128)
    fused(sh_out64, *sh64, 1)
    fused(sh_out128, *sh, 0)
    fused(sh_rnd, *[api.to_c128(x) for x in sh64], 0)
    torch.cuda.synchronize(dev)
    h64, h128, hr = sh_out64.cpu().numpy(), sh_out128.cpu().numpy(), sh_rnd.cpu().numpy()
    hrel, hin = np.abs(h64 - h128) / np.abs(h128), np.abs(hr - h128) / np.abs(h128)
    acc_signal["shifted_triple"] = {
        "inputs": "u - 1, u, u + 1 (the reference example's shifts of one propagator)",
        "max_rel_err_strict": float(hrel.max()), "median_rel_err_strict": float(np.median(hrel)),
        "input_rounding_only": {"max_rel_err_strict": float(hin.max()), "median_rel_err_strict": float(np.median(hin))},
        "max_rel_err_strict_first_16_timeslices": float(hrel[..., :16].max())}
    del sh, sh64

    # ---- e2e through the C ABI from pinned host complex128 buffers
    host = [x.cpu().pin_memory() for x in (u, u2, d)]
    host_out = torch.empty(out64.shape, dtype=out64.dtype).pin_memory()

    def e2e_step():
        # timeslice chunks copied back to back from the pinned host buffers on
        # one copy stream, converted and contracted as they arrive, correlators
        # copied back
        lib.contract_baryon_all_types_host(host_out.data_ptr(), *(h.data_ptr() for h in host), v, GAMMA_CG5,
                                           GAMMA_CG5, N_PROJ, proj_ptr, 1, latt_c)

    e2e_steps = max(1, min(args.steps, 5))
    ms_e2e, e2e_each = timed_each(e2e_step, e2e_steps, max(3, args.warmup))
    # the host link's own rate: plain pinned copies of the same three buffers
    scratch = torch.empty_like(host[0], device=dev)

    def link_step():
        for h in host:
            scratch.copy_(h, non_blocking=True)

    ms_link, link_each = timed_each(link_step, e2e_steps, max(3, args.warmup))
    del scratch
    e2e_err = float(np.abs(host_out.numpy() - out64.cpu().numpy()).max() / np.abs(out64.cpu().numpy()).max())
    ms_e2e = max_over_ranks(ms_e2e, world, dev)
    h2d = sum(x.numel() * x.element_size() for x in host)
    d2h = host_out.numel() * host_out.element_size()

    # ---- roofline of the dominant kernel (fused mixed): algorithmic bytes / time
    hbm_peak, peak_kind = peaks()
    bytes_per_launch = 3 * v * 1152 + N_TYPES * N_PROJ * lt * 16
    achieved = bytes_per_launch / (ms_mixed * 1e-3) / 1e9
    flops_per_launch = 8.0 * FUSED_CFMA_PER_SITE * v
    traffic = ncu_traffic()

    # ---- the other configurations of the path (one GPU): compact summaries
    configs = None
    if rank == 0 and world == 1 and not args.no_extra:
        ref_cpu = (sample_slices(u, args.cpu_slices), sample_slices(d, args.cpu_slices)) if not args.no_cpu else None
        del u2, u64, u264, d64, host, host_out
        torch.cuda.synchronize(dev)
        torch.cuda.empty_cache()
        env = (torch, lib, api, dev, stream)
        configs = {}
        for name, fn in (("C1_meson_8c16", workload_meson8), ("C3_momentum_32c64", workload_momentum32),
                         ("C4_sequential_48c96", workload_sequential48), ("C5_batch_mixed", workload_batch)):
            try:
                configs[name] = fn(args, env)
            except Exception as exc:  # reported, not hidden: the headline line still prints
                configs[name] = {"error": f"{type(exc).__name__}: {exc}"}
            torch.cuda.synchronize(dev)
            torch.cuda.empty_cache()
        lib.contract_set_stream(stream.cuda_stream)

    result = None
    if rank == 0:
        cb = None
        if not args.no_cpu:
            # the CPU leg contracts the first timeslices of the same u, d buffers;
            # its per-site values check both GPU forms on those timeslices
            ns = args.cpu_slices
            pu, pd = ref_cpu if configs is not None and ref_cpu else (sample_slices(u, ns), sample_slices(d, ns))
            cb, site = cpu_reference(1, 0, pu, pd)
            acc["vs_oracle"] = {"c128_fused": accuracy_vs_oracle(b, site, ns, 1e-12),
                                "c64_fused": accuracy_vs_oracle(a, site, ns, 1e-6),
                                "c64_fused_same_field": accuracy_vs_oracle(same_out, site, ns, 1e-6)}
            from oracle import lib as L
            oracle = L.ref_oracle() or L.c_oracle()
            pp = np.asarray(api.projector_plus_minus())
            ssite = np.array([[oracle.baryon_general_two_point(*sig_host, t, GAMMA_CG5, GAMMA_CG5, pp[w])
                               for w in range(N_PROJ)] for t in range(N_TYPES)])
            acc_signal["vs_oracle"] = {"c128_fused": accuracy_vs_oracle(sb, ssite, ns, 1e-12),
                                       "c64_fused": accuracy_vs_oracle(sa, ssite, ns, 1e-6)}
        ref_gpu = reference_gpu_leg(args)
        result = {
            "metric": METRIC, "value": value, "unit": "GSite/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_mixed, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64/f32 (f64 timeslice reduction)", "data": "synthetic",
            "config": workload_config(world),
            "hbm_gbs": achieved,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "traffic": traffic, "peak_source": peak_kind,
                         "kernel": fused_kernel_name(lib, v) + " + finalize_kernel",
                         "algorithmic_bytes_per_launch": bytes_per_launch},
            "fp32_pipe": {"achieved_tflops": flops_per_launch / (ms_mixed * 1e-3) / 1e12,
                          "peak_tflops": 73.1, "peak_source": "measured FFMA probe",
                          "frac": flops_per_launch / (ms_mixed * 1e-3) / 1e12 / 73.1},
            "plain_c128": {"fused_ms": ms_plain_fused, "fused_gsite_s": units / (ms_plain_fused * 1e-3) / 1e9,
                           "per_call_ms": ms_plain_call, "per_call_gsite_s": units / (ms_plain_call * 1e-3) / 1e9},
            "mixed_per_call": {"ms": ms_mixed_call, "gsite_s": units / (ms_mixed_call * 1e-3) / 1e9,
                               "hbm_gbs": 12 * 3 * v * 1152 / (ms_mixed_call * 1e-3) / 1e9},
            "speedup_mixed_vs_plain_per_call": ms_plain_call / ms_mixed,
            "mixed_same_field": {"ms": ms_same, "gsite_s": units / (ms_same * 1e-3) / 1e9,
                                 "max_diff_vs_two_buffers_rel_to_max": same_diff,
                                 "note": "u passed as P_i and P_j: one triangle pass (informational)"},
            "accuracy": acc,
            "accuracy_signal": acc_signal,
            "reference_gpu_c128": ref_gpu if not ref_gpu or "ms_per_call" not in ref_gpu else dict(
                ref_gpu, ours_plain_c128_per_call_ms=ms_plain_call / 12,
                speedup_ours_per_call=ref_gpu["ms_per_call"] / (ms_plain_call / 12),
                speedup_ours_fused_c128=ref_gpu["ms_per_sequence"] / ms_plain_fused,
                speedup_ours_mixed=ref_gpu["ms_per_sequence"] / ms_mixed),
            "e2e": {"value": world * units / (ms_e2e * 1e-3) / 1e9, "unit": "GSite/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": ms_e2e, "h2d_gbs": h2d / (ms_e2e * 1e-3) / 1e9,
                    "h2d_link_gbs": h2d / (ms_link * 1e-3) / 1e9, "frac_of_link": ms_link / ms_e2e,
                    # the host link is shared: a step that meets another tenant's traffic
                    # can take twice the others; value and ms_per_step keep every step
                    "ms_each_step": [round(x, 3) for x in e2e_each],
                    "ms_median_step": float(np.median(e2e_each)),
                    "value_from_median_step": world * units / (float(np.median(e2e_each)) * 1e-3) / 1e9,
                    "link_ms_each_step": [round(x, 3) for x in link_each],
                    "path": "contract_baryon_all_types_host (pinned complex128 in, chunked copy/convert/contract)",
                    "max_diff_vs_resident_rel_to_max": e2e_err},
            "gpu_launches": 2 * args.steps,
            "autotune": autotune_report(lib),
            "clocks": clocks.summary(),
            "cpu_baseline": None if cb is None else {k: cb[k] for k in ("value", "unit", "cores", "cpu_model", "kind",
                                                                          "sample")},
            "configs": configs,
        }
        print(json.dumps(result), flush=True)
    return result


# ------------------------------------------------------- other workloads --
# The other configurations of the path, each returning a compact summary that
# the default run attaches to its JSON line ("configs") and that
# ``--workload NAME`` prints alone.

def _gpu_env():
    import torch

    from contract_gb300 import _lib, api, build
    build.build()
    lib = _lib.lib()
    lib.contract_set_error_mode(1)
    lib.contract_set_autotune(1)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    lib.contract_set_stream(stream.cuda_stream)
    return torch, lib, api, dev, stream


def _time(torch, stream, fn, steps, warmup, lib):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    e1.synchronize()
    if lib.contract_last_error():
        raise RuntimeError(lib.contract_last_error_message().decode())
    return e0.elapsed_time(e1) / steps


def _rel(a, b, sigma=None):
    """Strict relative error |a - b| / |b| and, given the spread sigma of the
    site values behind each sum, the sigma-normalised |a - b| / max(|b|, sigma)."""
    d = np.abs(a - b)
    r = d / np.maximum(np.abs(b), 1e-300)
    out = {"max_rel_err_strict": float(r.max()), "median_rel_err_strict": float(np.median(r)),
           "frac_le_1e-6_strict": float((r <= 1e-6).mean()), "pass_strict_1e-6": bool(r.max() <= 1e-6),
           "max_err_rel_to_max": float(d.max() / np.abs(b).max())}
    if sigma is not None:
        n = d / np.maximum(np.abs(b), sigma)
        out.update({"max_rel_err_sigma_normalised": float(n.max()), "pass_sigma_normalised_1e-6": bool(n.max() <= 1e-6)})
    return out


def _moms(nmax):
    r = np.arange(-nmax, nmax + 1)
    m = np.ascontiguousarray(np.stack(np.meshgrid(r, r, r, indexing="ij"), -1).reshape(-1, 3)[:, ::-1].astype(np.int32))
    return m, m.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _pair_sigma(torch, lib, p1, p2, latt):
    """sigma_t of every meson pair: sqrt(sum_{x in t} |C_ab(x)|^2) [Lt, 256] from
    the complex128 per-site values (16 meson_all_source calls, per site)."""
    v = p1.shape[0]
    out = torch.empty((16, 16, v), dtype=torch.complex128, device=p1.device)
    for a in range(16):
        ptrs = (ctypes.c_void_p * 16)(*[out[a, k].data_ptr() for k in range(16)])
        lib.contract_meson_all(ptrs, p1.data_ptr(), p2.data_ptr(), v, a, 1, 0, None)
    sq = (out.abs() ** 2).reshape(256, 2, latt[3], -1).sum(dim=(1, 3))
    return sq.sqrt().T.cpu().numpy()  # [Lt, 256]


def _product_l1(torch, p1, p2, latt):
    """Error scale of a momentum projection with one field in both slots:
    per timeslice, the largest sum_x |T(x)| over the 256 spin-colour products
    T[i][j][k][l](x) = sum_c S1[i][k][c] conj(S2[j][l][c]) [1, Lt, 1]: the
    diagonal products are then positive at every site, and at nonzero momentum
    an FP32 projection cancels terms of this size (complex128 arithmetic on the
    device, in chunks of sites)."""
    v = p1.shape[0]
    a, b = p1.reshape(v, 4, 4, 9), p2.reshape(v, 4, 4, 9)
    per_site = torch.empty((v, 256), dtype=torch.float64, device=p1.device)
    step = 1 << 18
    for s0 in range(0, v, step):
        t = torch.einsum("xikc,xjlc->xijkl", a[s0:s0 + step], b[s0:s0 + step].conj())
        per_site[s0:s0 + step] = t.abs().reshape(-1, 256)
    l1 = per_site.reshape(2, latt[3], -1, 256).sum(dim=(0, 2)).max(dim=1).values
    return l1.cpu().numpy()[None, :, None]


def _cudart():
    """The CUDA runtime library the process has loaded (for graph inspection)."""
    for line in open("/proc/self/maps"):
        if "libcudart.so" in line:
            return ctypes.CDLL(line.split()[-1])
    return None


def graph_kernel_nodes(lib, fn):
    """Kernel launches in a CUDA graph captured from fn() (after a warm-up
    call): the launches one step of fn makes.  None if the runtime's graph
    calls are not reachable."""
    rt = _cudart()
    if rt is None:
        return None
    vp = ctypes.c_void_p
    stream, graph = vp(), vp()
    if rt.cudaStreamCreate(ctypes.byref(stream)) != 0:
        return None
    old = lib.contract_get_stream()
    try:
        lib.contract_set_stream(stream)
        if rt.cudaStreamBeginCapture(stream, 1) != 0:  # cudaStreamCaptureModeThreadLocal
            return None
        fn()
        if rt.cudaStreamEndCapture(stream, ctypes.byref(graph)) != 0:
            return None
        n = ctypes.c_size_t(0)
        rt.cudaGraphGetNodes(graph, None, ctypes.byref(n))
        nodes = (vp * n.value)()
        rt.cudaGraphGetNodes(graph, nodes, ctypes.byref(n))
        kinds = [ctypes.c_int(0) for _ in range(n.value)]
        for node, k in zip(nodes, kinds):
            rt.cudaGraphNodeGetType(vp(node), ctypes.byref(k))
        rt.cudaGraphDestroy(graph)
        return sum(1 for k in kinds if k.value == 0)  # cudaGraphNodeTypeKernel
    finally:
        lib.contract_set_stream(old)
        rt.cudaStreamSynchronize(stream)
        rt.cudaStreamDestroy(stream)


def workload_meson8(args, env=None):
    """8^3 x 16: all 16 x 16 meson correlators at zero momentum (two complex128
    propagators, m = 0.3), through the drop-in meson_all_source_two_point (16
    calls, per site, complex128) and the fused complex64 projection; against
    the C oracle's per-site values."""
    torch, lib, api, dev, stream = env or _gpu_env()
    from contract_gb300.lattice import synthetic_propagator
    from oracle import einsum_oracle as eo
    latt = (8, 8, 8, 16)
    v = latt[0] * latt[1] * latt[2] * latt[3]
    p1 = synthetic_propagator(latt, 41, 0.3, device=dev)
    p2 = synthetic_propagator(latt, 42, 0.3, device=dev)
    q1, q2 = api.to_c64(p1), api.to_c64(p2)
    site = torch.empty((16, 16, v), dtype=torch.complex128, device=dev)

    def dropin():
        for a in range(16):
            ptrs = (ctypes.c_void_p * 16)(*[site[a, k].data_ptr() for k in range(16)])
            lib.meson_all_source_two_point(ptrs, p1.data_ptr(), p2.data_ptr(), v, a)

    ms_dropin = _time(torch, stream, dropin, 20, 3, lib)
    m0 = np.zeros((1, 3), dtype=np.int32)
    out64 = torch.empty((1, latt[3], 256), dtype=torch.complex128, device=dev)
    lat = (ctypes.c_int * 4)(*latt)
    ms_mom = _time(torch, stream, lambda: lib.contract_meson_all_gamma_momentum(
        out64.data_ptr(), q1.data_ptr(), q2.data_ptr(), v, lat, m0.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), 1, 1),
        20, 3, lib)
    torch.cuda.synchronize()
    # the oracle's per-site values: the meson all-gamma restatement on the host
    ref_site = eo.meson_all_gamma(p1.cpu().numpy(), p2.cpu().numpy()).reshape(256, -1)
    got_site = site.reshape(256, -1).cpu().numpy()
    ref_t = eo.timeslice_sum(ref_site, latt).T  # [Lt, 256]
    sig = np.sqrt(eo.timeslice_sum(np.abs(ref_site) ** 2, latt).real).T
    return {"workload": "meson_8c16", "lattice": list(latt), "pairs": 256, "momenta": 1,
            "dropin_c128_ms": ms_dropin, "dropin_c128_gsite_s": v * 256 / ms_dropin / 1e6,
            "fused_c64_ms": ms_mom, "fused_c64_gsite_s": v * 256 / ms_mom / 1e6,
            "accuracy": {"dropin_c128_vs_oracle_per_site": float(np.abs(got_site - ref_site).max()
                                                                  / np.abs(ref_site).max()),
                         "fused_c64_vs_oracle": _rel(out64[0].cpu().numpy(), ref_t, sig)}}


def workload_momentum32(args, env=None):
    """All 16 x 16 meson pairs at 125 momenta on 32^3 x 64."""
    torch, lib, api, dev, stream = env or _gpu_env()
    from contract_gb300.lattice import synthetic_propagator
    latt = (32, 32, 32, 64)
    v = latt[0] * latt[1] * latt[2] * latt[3]
    steps = max(1, min(args.steps, 20))
    p1 = synthetic_propagator(latt, 11, 0.2, device=dev)
    p2 = synthetic_propagator(latt, 12, 0.2, device=dev)
    q1, q2 = api.to_c64(p1), api.to_c64(p2)
    moms, mp = _moms(2)
    lat = (ctypes.c_int * 4)(*latt)
    out64 = torch.empty((len(moms), latt[3], 256), dtype=torch.complex128, device=dev)
    out128 = torch.empty_like(out64)
    with ClockSampler(0) as clocks:
        ms64 = _time(torch, stream, lambda: lib.contract_meson_all_gamma_momentum(
            out64.data_ptr(), q1.data_ptr(), q2.data_ptr(), v, lat, mp, len(moms), 1), steps, 3, lib)
    outtc = torch.empty_like(out64)
    ms_tc = _time(torch, stream, lambda: lib.contract_meson_all_gamma_momentum(
        outtc.data_ptr(), q1.data_ptr(), q2.data_ptr(), v, lat, mp, len(moms), 2), steps, 3, lib)
    ms128 = _time(torch, stream, lambda: lib.contract_meson_all_gamma_momentum(
        out128.data_ptr(), p1.data_ptr(), p2.data_ptr(), v, lat, mp, len(moms), 0), 2, 1, lib)
    # one field passed twice (a pion): Hermitian site products; against the
    # general form on a copy of the field
    out_same, out_copy = torch.empty_like(out64), torch.empty_like(out64)
    ms_same = _time(torch, stream, lambda: lib.contract_meson_all_gamma_momentum(
        out_same.data_ptr(), q1.data_ptr(), q1.data_ptr(), v, lat, mp, len(moms), 1), steps, 3, lib)
    q1c = q1.clone()
    ms_copy = _time(torch, stream, lambda: lib.contract_meson_all_gamma_momentum(
        out_copy.data_ptr(), q1.data_ptr(), q1c.data_ptr(), v, lat, mp, len(moms), 1), steps, 3, lib)
    a_same, a_copy = out_same.cpu().numpy(), out_copy.cpu().numpy()
    del q1c, out_same, out_copy
    sig = _pair_sigma(torch, lib, p1, p2, latt)[None]  # [1, Lt, 256]
    units = v * 256
    dense_flop = 8.0 * len(moms) * 256 * v  # the per-timeslice dense complex GEMM
    hbm = peaks()[0]
    ref = out128.cpu().numpy()
    return {"workload": "momentum32", "lattice": list(latt), "momenta": len(moms), "pairs": 256,
            "mixed_ms": ms64, "tensor_ms": ms_tc, "plain_ms": ms128, "mixed_gsite_s": units / ms64 / 1e6,
            "tensor_gsite_s": units / ms_tc / 1e6, "plain_gsite_s": units / ms128 / 1e6,
            "speedup": ms128 / ms64, "speedup_tensor": ms128 / ms_tc,
            "mixed_hbm_frac": 2 * v * 1152 / (ms64 * 1e-3) / 1e9 / hbm,
            "dense_gemm_equiv_tflops_mixed": dense_flop / ms64 / 1e9,
            "dense_gemm_equiv_tflops_tensor": dense_flop / ms_tc / 1e9,
            "accuracy_mixed_vs_plain": _rel(out64.cpu().numpy(), ref, sig),
            "accuracy_tensor_vs_plain": _rel(outtc.cpu().numpy(), ref, sig),
            "same_field": {"ms": ms_same, "general_form_on_a_copy_ms": ms_copy,
                           "max_diff_rel_to_max": float(np.abs(a_same - a_copy).max() / np.abs(a_copy).max())},
            "clocks": clocks.summary()}


def workload_sequential48(args, env=None):
    """On 48^3 x 96: the sequential source (full volume, and
    the t_sink = 24 insertion with zeros elsewhere), then a zero-momentum
    baryon_general two-point with (1 + g4)/2; complex128 vs complex64 storage
    of the same propagator values."""
    torch, lib, api, dev, stream = env or _gpu_env()
    from contract_gb300.lattice import synthetic_propagator
    latt = (48, 48, 48, 96)
    v = latt[0] * latt[1] * latt[2] * latt[3]
    steps = max(1, min(args.steps, 10))
    lat = (ctypes.c_int * 4)(*latt)
    pp = np.ascontiguousarray(api.projector_plus_minus())
    hbm = peaks()[0]
    res = {"workload": "sequential48", "lattice": list(latt), "t_sink": 24, "type": "IK_JL_NM",
           "sequential": "SEQUENTIAL_N (writes propag_n)", "gamma": "C g5, C g5, (1 + g4)/2"}
    u128 = synthetic_propagator(latt, 21, 0.25, device=dev)
    d128 = synthetic_propagator(latt, 23, 0.30, device=dev)
    seq128 = torch.empty_like(u128)
    kept = {}
    clocks = ClockSampler(0)
    for name, prec in (("c128", 0), ("c64", 1)):
        u, d = (u128, d128) if prec == 0 else (api.to_c64(u128), api.to_c64(d128))
        seq = seq128 if prec == 0 else torch.empty_like(u)
        corr = torch.empty(latt[3], dtype=torch.complex128, device=dev)
        site = 1152 if prec else 2304
        st = steps if prec else 2
        if prec:
            clocks.__enter__()
        ms_full = _time(torch, stream, lambda: lib.contract_sequential(
            u.data_ptr(), u.data_ptr(), seq.data_ptr(), 0, 2, v, 5, 5, 8, prec), st, 1, lib)
        ms_sink = _time(torch, stream, lambda: lib.contract_sequential_sink(
            u.data_ptr(), u.data_ptr(), seq.data_ptr(), 0, 2, v, lat, 24, 5, 5, 8, prec), st, 1, lib)
        ms_2pt = _time(torch, stream, lambda: lib.contract_baryon(
            corr.data_ptr(), u.data_ptr(), u.data_ptr(), d.data_ptr(), 0, v, 5, 5, 0, pp[0].ctypes.data, prec, lat),
            st, 1, lib)
        if prec:
            clocks.__exit__(None, None, None)
        slab = seq.view(2, latt[3], -1)[:, 24].to(torch.complex128)
        kept[name] = (corr.cpu().numpy(), slab)
        res[name] = {"sequential_full_ms": ms_full, "sequential_full_gbs": 3 * v * site / ms_full / 1e6,
                     "sequential_full_hbm_frac": 3 * v * site / ms_full / 1e6 / hbm,
                     "sequential_full_gsite_s": v / ms_full / 1e6,
                     "sequential_sink_ms": ms_sink, "sequential_sink_write_gbs": v * site / ms_sink / 1e6,
                     "twopt_ms": ms_2pt, "twopt_gbs": 3 * v * site / ms_2pt / 1e6,
                     "twopt_hbm_frac": 3 * v * site / ms_2pt / 1e6 / hbm, "twopt_gsite_s": v / ms_2pt / 1e6}
        if prec:
            del u, d, seq
            torch.cuda.empty_cache()
    # sigma_t of the two-point from its complex128 per-site values
    per_site = torch.empty(v, dtype=torch.complex128, device=dev)
    lib.contract_baryon(per_site.data_ptr(), u128.data_ptr(), u128.data_ptr(), d128.data_ptr(), 0, v, 5, 5, 0,
                        pp[0].ctypes.data, 0, None)
    sig = (per_site.abs() ** 2).reshape(2, latt[3], -1).sum(dim=(0, 2)).sqrt().cpu().numpy()
    del per_site, u128, d128, seq128
    torch.cuda.empty_cache()
    c128, s128 = kept["c128"]
    c64, s64 = kept["c64"]
    res["speedup_c64_vs_c128"] = {k: res["c128"][k] / res["c64"][k] for k in
                                  ("sequential_full_ms", "sequential_sink_ms", "twopt_ms")}
    res["accuracy_c64_vs_c128"] = {
        "twopt": _rel(c64, c128, sig),
        "sink_slab_max_err_rel_to_max": float((s64 - s128).abs().max() / s128.abs().max())}
    res["clocks"] = clocks.summary()
    return res


class _MesonItem(ctypes.Structure):
    _fields_ = [("propag_i", ctypes.c_void_p), ("propag_j", ctypes.c_void_p), ("correl", ctypes.c_void_p),
                ("lattice", ctypes.c_int * 4)]


class _BaryonItem(ctypes.Structure):
    _fields_ = [("propag_i", ctypes.c_void_p), ("propag_j", ctypes.c_void_p), ("propag_n", ctypes.c_void_p),
                ("correl", ctypes.c_void_p), ("lattice", ctypes.c_int * 4)]


def workload_batch(args, env=None):
    """64 sources on 16^3x32, 24^3x48 and 32^3x64 lattices,
    each with the 16 x 16 meson at 27 momenta and all baryon types, through
    contract_batch_mixed: one persistent baryon launch, one persistent meson
    launch and one finalisation, captured in a CUDA graph, complex64; the
    baryon and meson batches are also timed alone; compared with the plain
    per-call FP64 form on one source per lattice."""
    torch, lib, api, dev, stream = env or _gpu_env()
    from contract_gb300.lattice import synthetic_propagator
    classes = [((16, 16, 16, 32), 24), ((24, 24, 24, 48), 24), ((32, 32, 32, 64), 16)]
    rng = np.random.default_rng(5)
    moms, mp = _moms(1)
    pp = np.ascontiguousarray(api.projector_plus_minus())
    steps = max(1, min(args.steps, 10))
    sources = []
    seed = 1000
    for latt, count in classes:
        for _ in range(count):
            mu, md = rng.uniform(0.1, 0.5, 2)
            u = synthetic_propagator(latt, seed, float(mu), device=dev, dtype=torch.complex64)
            d = synthetic_propagator(latt, seed + 1, float(md), device=dev, dtype=torch.complex64)
            seed += 2
            sources.append({"latt": latt, "u": u, "d": d, "mu": float(mu), "md": float(md),
                            "bary": torch.empty((6, 2, latt[3]), dtype=torch.complex128, device=dev),
                            "mes": torch.empty((len(moms), latt[3], 256), dtype=torch.complex128, device=dev)})
    n = len(sources)
    bitems, mitems = (_BaryonItem * n)(), (_MesonItem * n)()
    for k, s in enumerate(sources):
        bitems[k].propag_i = bitems[k].propag_j = s["u"].data_ptr()
        bitems[k].propag_n = s["d"].data_ptr()
        bitems[k].correl = s["bary"].data_ptr()
        bitems[k].lattice = (ctypes.c_int * 4)(*s["latt"])
        mitems[k].propag_i = mitems[k].propag_j = s["u"].data_ptr()
        mitems[k].correl = s["mes"].data_ptr()
        mitems[k].lattice = (ctypes.c_int * 4)(*s["latt"])

    def step():
        lib.contract_batch_mixed(bitems, n, 5, 5, 2, pp.ctypes.data, mitems, n, mp, len(moms), 1)

    def baryon_only():
        lib.contract_baryon_all_types_batch(bitems, n, 5, 5, 2, pp.ctypes.data, 1)

    def meson_only():
        lib.contract_meson_all_gamma_momentum_batch(mitems, n, mp, len(moms), 1)

    def graph_of(fn):
        fn()  # autotune (per extent) and workspace growth before capture
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            lib.contract_set_stream(torch.cuda.current_stream().cuda_stream)
            fn()
        lib.contract_set_stream(stream.cuda_stream)
        return g

    step()  # autotune (per extent) and workspace growth happen before any capture
    torch.cuda.synchronize()
    launches = graph_kernel_nodes(lib, step)
    gb, gm = graph_of(baryon_only), graph_of(meson_only)
    ms_baryon = _time(torch, stream, gb.replay, steps, 2, lib)
    ms_meson = _time(torch, stream, gm.replay, steps, 2, lib)
    del gb, gm
    g = graph_of(step)
    with ClockSampler(0) as clocks:
        ms_graph = _time(torch, stream, g.replay, steps, 2, lib)
    sites = sum(s["u"].numel() // 144 for s in sources)
    # plain per-call FP64 on the first source of each lattice class, extrapolated by site count
    plain_ms_total, errs = 0.0, []
    first = 0
    for latt, count in classes:
        s = sources[first]
        first += count
        u, d = s["u"].to(torch.complex128), s["d"].to(torch.complex128)
        vs = u.numel() // 144
        lat = (ctypes.c_int * 4)(*latt)
        bary = torch.empty((6, 2, latt[3]), dtype=torch.complex128, device=dev)
        mes = torch.empty_like(s["mes"])

        def plain():
            for t in range(6):
                for w in range(2):
                    lib.contract_baryon(bary[t, w].data_ptr(), u.data_ptr(), u.data_ptr(), d.data_ptr(), t, vs, 5, 5, 0,
                                        pp[w].ctypes.data, 0, lat)
            lib.contract_meson_all_gamma_momentum(mes.data_ptr(), u.data_ptr(), u.data_ptr(), vs, lat, mp, len(moms), 0)

        plain_ms_total += _time(torch, stream, plain, 1, 1, lib) * count
        # sigma_t from the complex128 per-site values
        site = torch.empty((6, 2, vs), dtype=torch.complex128, device=dev)
        lib.contract_baryon_all_types(site.data_ptr(), u.data_ptr(), u.data_ptr(), d.data_ptr(), vs, 5, 5, 2,
                                      pp.ctypes.data, 0, None)
        bsig = (site.abs() ** 2).reshape(6, 2, 2, latt[3], -1).sum(dim=(2, 4)).sqrt().cpu().numpy()
        del site
        # one field in both meson slots: the scale is the products' L1 (see _product_l1)
        msig = np.maximum(_pair_sigma(torch, lib, u, u, latt)[None], _product_l1(torch, u, u, latt))
        errs.append({"lattice": list(latt), "baryon": _rel(s["bary"].cpu().numpy(), bary.cpu().numpy(), bsig),
                     "meson": _rel(s["mes"].cpu().numpy(), mes.cpu().numpy(), msig),
                     "meson_scale": "max(|C|, sigma, L1): one field in both slots"})
        del u, d
    baryon_units, meson_units = sites * 12, sites * 256 * len(moms)
    res = {"workload": "batch", "sources": n, "site_sources": sites,
           "contractions_per_site": {"baryon": 12, "meson_pairs": 256, "momenta": len(moms)},
           "mixed_graph_ms": ms_graph, "kernel_launches_per_step": launches,
           "baryon_batch_ms": ms_baryon, "baryon_gsite_s": baryon_units / ms_baryon / 1e6,
           "baryon_hbm_gbs": sites * 2 * 1152 / ms_baryon / 1e6,
           "meson_batch_ms": ms_meson, "meson_gsite_pair_s": sites * 256 / ms_meson / 1e6,
           "meson_hbm_gbs": sites * 1152 / ms_meson / 1e6,
           "plain_per_call_ms_extrapolated": plain_ms_total, "speedup": plain_ms_total / ms_graph,
           "note": ("P_i = P_j = u in every item, so the mixed form takes the one-pass baryon and the Hermitian meson "
                    "products; the plain per-call baseline does the general work"),
           "accuracy_mixed_vs_plain": errs, "autotune": [r for r in autotune_report(lib) if "batch=" in r[0]],
           "clocks": clocks.summary()}
    del g, sources
    torch.cuda.empty_cache()
    return res


WORKLOADS = {"meson8": workload_meson8, "momentum32": workload_momentum32, "sequential48": workload_sequential48,
             "batch": workload_batch}


PROFILE_OPS = ("fused", "fused128", "fused1", "fused1128", "fusedsame", "tri", "tri128", "trigen", "trigen128", "tridense", "tridense128",
               "loop", "loop128", "loopgen", "loopgen128", "momentum",
               "momentum128", "momentum_tc", "meson", "meson128", "meson_all",
               "diquark", "sequential", "sequential128", "batch_mixed")


def autotune_report(lib):
    buf = ctypes.create_string_buffer(8192)
    lib.contract_autotune_report(buf, len(buf))
    return [line.split("\t") for line in buf.value.decode().splitlines()]


def run_profile(args):
    """One op, nothing else: the command line that ncu captures (small lattice)."""
    import torch

    from contract_gb300 import _lib, api, build
    from contract_gb300.lattice import synthetic_propagator

    build.build()
    lib = _lib.lib()
    lib.contract_set_error_mode(1)
    lib.contract_set_autotune(0 if args.no_autotune else 1)
    latt = tuple(int(x) for x in args.lattice.split(","))
    v = latt[0] * latt[1] * latt[2] * latt[3]
    dev = torch.device("cuda", 0)
    lib.contract_set_stream(torch.cuda.current_stream(dev).cuda_stream)
    op = args.profile
    c64 = not op.endswith("128")
    base = op[:-3] if op.endswith("128") else op
    props = [synthetic_propagator(latt, s, m, device=dev) for s, m in ((1, 0.25), (2, 0.25), (3, 0.30))]
    if c64:
        props = [api.to_c64(p) for p in props]
    prec = 1 if c64 else 0
    latt_c = (ctypes.c_int * 4)(*latt)
    projs = np.ascontiguousarray(api.projector_plus_minus())
    rng = np.random.default_rng(5)
    dense = np.ascontiguousarray((rng.standard_normal(16) + 1j * rng.standard_normal(16)) / 4)
    out = torch.empty((16, max(v, 1)), dtype=torch.complex128, device=dev)
    field = torch.empty_like(props[0])
    a, b_, c = (x.data_ptr() for x in props)
    r = np.arange(-2, 3)
    moms = np.ascontiguousarray(np.stack(np.meshgrid(r, r, r, indexing="ij"), -1).reshape(-1, 3)[:, ::-1]
                                .astype(np.int32))
    moms_ptr = moms.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    mom_out = torch.empty((len(moms), latt[3], 256), dtype=torch.complex128, device=dev) \
        if base.startswith("momentum") else None
    if base == "batch_mixed":  # four sources on the lattice: baryon and meson (27 momenta) items, one mixed call
        m27, mp27 = _moms(1)
        nb = 4
        bsrc = [(props[0], props[2])] + [(synthetic_propagator(latt, 10 + k, 0.2, device=dev, dtype=torch.complex64),
                                          synthetic_propagator(latt, 20 + k, 0.3, device=dev, dtype=torch.complex64))
                                         for k in range(nb - 1)]
        b_out = [torch.empty((6, 2, latt[3]), dtype=torch.complex128, device=dev) for _ in range(nb)]
        m_out = [torch.empty((len(m27), latt[3], 256), dtype=torch.complex128, device=dev) for _ in range(nb)]
        bitems, mitems = (_BaryonItem * nb)(), (_MesonItem * nb)()
        for k, (uu, dd) in enumerate(bsrc):
            bitems[k].propag_i = bitems[k].propag_j = mitems[k].propag_i = mitems[k].propag_j = uu.data_ptr()
            bitems[k].propag_n = dd.data_ptr()
            bitems[k].correl, mitems[k].correl = b_out[k].data_ptr(), m_out[k].data_ptr()
            bitems[k].lattice = mitems[k].lattice = (ctypes.c_int * 4)(*latt)

    def step():
        if base == "fused":
            lib.contract_baryon_all_types(out.data_ptr(), a, b_, c, v, 5, 5, 2, projs.ctypes.data, prec, latt_c)
        elif base == "fused1":  # one projector, (1 + g4)/2 (rank 2: the factored triangles)
            lib.contract_baryon_all_types(out.data_ptr(), a, b_, c, v, 5, 5, 1, projs.ctypes.data, prec, latt_c)
        elif base == "fusedsame":  # one field passed as P_i and P_j
            lib.contract_baryon_all_types(out.data_ptr(), a, a, c, v, 5, 5, 2, projs.ctypes.data, prec, latt_c)
        elif base in ("tri", "loop"):  # baryon_two_point form: Gamma_mn = g4
            lib.contract_baryon(out.data_ptr(), a, b_, c, 1 if base == "tri" else 0, v, 5, 5, 8, None, prec, latt_c)
        elif base == "trigen":  # general projector (1 + g4)/2 (rank 2: the factored form)
            lib.contract_baryon(out.data_ptr(), a, b_, c, 1, v, 5, 5, 0, projs[0].ctypes.data, prec, latt_c)
        elif base == "loopgen":  # loop form (type 0) with the general projector (1 + g4)/2
            lib.contract_baryon(out.data_ptr(), a, b_, c, 0, v, 5, 5, 0, projs[0].ctypes.data, prec, latt_c)
        elif base == "tridense":  # a dense projector (rank 4: N' = W N per site)
            lib.contract_baryon(out.data_ptr(), a, b_, c, 1, v, 5, 5, 0, dense.ctypes.data, prec, latt_c)
        elif base == "meson":
            lib.contract_meson(out.data_ptr(), a, b_, v, 15, 15, prec, latt_c)
        elif base == "meson_all":
            ptrs = (ctypes.c_void_p * 16)(*[out[k].data_ptr() for k in range(16)])
            lib.contract_meson_all(ptrs, a, b_, v, 5, 1, prec, latt_c)
        elif base == "diquark":
            lib.contract_diquark(field.data_ptr(), a, b_, v, 5, 5, prec)
        elif base == "momentum":  # all 16 x 16 meson pairs at the 125 momenta n in {-2..2}^3
            lib.contract_meson_all_gamma_momentum(mom_out.data_ptr(), a, b_, v, latt_c, moms_ptr, len(moms), prec)
        elif base == "momentum_tc":  # the same on the tensor cores (split bf16)
            lib.contract_meson_all_gamma_momentum(mom_out.data_ptr(), a, b_, v, latt_c, moms_ptr, len(moms), 2)
        elif base == "sequential":
            lib.contract_sequential(a, b_, c, 1, 2, v, 5, 5, 8, prec)
        elif base == "batch_mixed":
            lib.contract_batch_mixed(bitems, nb, 5, 5, 2, projs.ctypes.data, mitems, nb, mp27, len(m27), 1)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    e1.synchronize()
    if lib.contract_last_error():
        raise RuntimeError(lib.contract_last_error_message().decode())
    print(json.dumps({"profile": op, "lattice": list(latt), "ms_per_launch": e0.elapsed_time(e1) / args.steps,
                      "autotune": autotune_report(lib)}))


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--cpu-slices", type=int, default=8, help="timeslices in the CPU baseline sample")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-ref-gpu", action="store_true", help="skip timing the reference's own GPU kernels")
    ap.add_argument("--no-autotune", action="store_true", help="use the default tile shapes")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the other configurations (8^3x16 meson, 32^3x64 momentum, 48^3x96 sequential, batch)")
    ap.add_argument("--profile", choices=PROFILE_OPS, help="run only this op (for ncu captures)")
    ap.add_argument("--lattice", default="24,24,24,16", help="Lx,Ly,Lz,Lt for --profile")
    ap.add_argument("--workload", choices=sorted(WORKLOADS),
                    help="measure one other configuration alone (meson 8^3x16, momentum projection, sequential source, batch)")
    args = ap.parse_args()
    if args.profile:
        run_profile(args)
        return
    if args.workload:
        print(json.dumps(WORKLOADS[args.workload](args)), flush=True)
        return
    world, rank, local = dist_setup(args)
    try:
        if args.impl == "reference":
            run_reference(args, world, rank)
        else:
            run_ours(args, world, rank, local)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
