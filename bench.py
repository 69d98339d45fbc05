"""Benchmark: MT forward solves per second on the 256x256x48 precision model.

One step is one MT solve at one frequency: the Green tensor built in FP64 on
the device (stored complex64 for the inner solver and complex128 for the
refinement residual), both polarisations solved to a 1e-6 relative true
residual by the mixed-precision solve (complex64 FGMRES with a GMRES
preconditioner inside FP64 iterative refinement), then E and H at the
surface (level tensors built in FP64) and the impedance, apparent
resistivity and phase at all 256x256 cell centres. Steps cycle over the
model's four frequencies (1e-3 .. 10 Hz, log-spaced).

Keys of the JSON line beyond the common ones:
  e2e          the same solves through the C ABI with host buffers
               (zeta, zeta0, dz, E0 copied in; surface E and H of both
               polarisations out);
  roofline     the complex64 block-contraction kernel, its CUDA-event time on
               the library's stream during the timed region, against the
               measured HBM copy bandwidth;
  plain_fp64   one solve of the reference algorithm (complex128 FGMRES with
               the reference's defaults) at the second frequency, beside the
               timed mixed step at that frequency;
  cpu_baseline the numpy/scipy restatement timed on this host's cores on a
               bounded sample (one operator apply), scaled to a solve.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With N > 1 every rank solves its own seeded model on its own GPU (replicas;
the path has no exchange step).
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

METRIC = "MT solves/s to 1e-6 residual (256x256x48): mixed+learned vs plain FP64, 1 GB300"

# DRAM bytes (read + write) of one launch of the complex64 contraction at
# 256x256x48, by right-hand sides per launch, measured by ncu at 128x128x48
# (16,641 stored points) and scaled by the algorithmic bytes, which grow with
# the stored points. One: 1.4262 GB x 5.6765 / 1.4290; two (k_contract_sb3):
# 1.5719 GB x 6.2805 / 1.5800.
CONTRACT_TRAFFIC_BYTES = {1: 5.665e9, 2: 6.248e9}

# Operator applications per polarisation of the reference algorithm
# (complex128 FGMRES(15) with GMRES(10), tolerance 1e-6) on the 256x256x48
# model: the reference arm turns its timed apply into a solve with it.
REFERENCE_APPLIES_PER_POL = 170


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=4)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="precision", choices=["precision", "medium", "small", "batching"],
                   help="batching: the 64-solve configuration of uneven meshes (concurrent streams, tuned count)")
    p.add_argument("--mesh", default=None, help="NXxNYxNZ: the same generator at another mesh (profiling cases)")
    p.add_argument("--no-plain", action="store_true", help="skip the plain FP64 solve")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    p.add_argument("--no-batch", action="store_true",
                   help="solve the two polarisations one after the other instead of as one stacked system")
    return p.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def make_model(workload, seed, mesh=None):
    from extreme_gb300.model import medium_model, precision_model, scaled_model, small_model
    if mesh:
        nx, ny, nz = (int(v) for v in mesh.lower().split("x"))
        return scaled_model(nx, ny, nz, seed)
    if workload == "precision":
        return precision_model(seed)
    if workload == "medium":
        return medium_model(seed)
    return small_model()


def c64_block_entries(nz):
    """Complex entries of one stored spectral point of the complex64 Green
    copy: 4x4 sub-blocks (upper triangle of xx, xy, yy, zz; all of xz, yz)
    for nz in {16, 32, 48}, else packed triangles + row-padded xz, yz."""
    if nz in (16, 32, 48):
        nb = nz // 4
        return 4 * nb * (nb + 1) // 2 * 16 + 2 * nb * nb * 16
    return 4 * (nz * (nz + 1) // 2) + 2 * nz * (nz + 1)


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    REASONS = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        threading.Thread(target=self._read, daemon=True).start()

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
        sm, smax, power, reasons = [], [], [], set()
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for name, val in zip(self.REASONS, f[5:9]):
                if val.lower() in ("active", "1"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- our arm
def job_rate(ms_total, ms_e2e, steps, world, device="cpu"):
    """Replicas: every rank timed `steps` solves of its own model. The job's
    time is the slowest rank's (max over ranks, on `device` for the process
    group's backend); its rate counts every rank's solves. Returns
    (max ms, max e2e ms, whole-job solves/s)."""
    ms_max, e2e_max = ms_total, ms_e2e
    if world > 1:
        import torch
        import torch.distributed as tdist
        t = torch.tensor([ms_total, ms_e2e], dtype=torch.float64, device=device)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        ms_max, e2e_max = float(t[0]), float(t[1])
    return ms_max, e2e_max, steps * world / (ms_max / 1e3)


def run_ours(args, rank, world, local):
    import torch

    from extreme_gb300 import egx
    from extreme_gb300.forward import model_zeta
    from extreme_gb300.model import freq_to_omega

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    m = make_model(args.workload, seed=1 + rank, mesh=args.mesh)
    freqs = list(m.frequencies)
    nf = len(freqs)
    ctx = egx.Context(local)
    # the library launches on this stream, so events recorded on it time its kernels
    stream = torch.cuda.Stream(dev)
    ctx.set_stream(stream.cuda_stream)
    # every step builds its level tensors like a fresh solve: no reuse across steps
    ctx.level_cache(0)
    n = m.nx * m.ny * 3 * m.nz
    mixed = dict(tol=1e-6, max_outer=5, m_out=30, m_in=10, inner_tol=5e-7, inner_restarts=20,
                 batch=not args.no_batch)

    host_in, host_e0 = [], []
    for f in freqs:
        omega = freq_to_omega(f)
        host_in.append(model_zeta(m, omega))
        host_e0.append(np.ascontiguousarray(np.stack([egx.normal_field(m, omega)] * 2)))
    zeta_d = [torch.from_numpy(z.reshape(-1).view(np.float64)).to(dev) for z, _ in host_in]
    zeta0_d = [torch.from_numpy(z0.view(np.float64)).to(dev) for _, z0 in host_in]
    e0_d = [torch.from_numpy(e.reshape(-1).view(np.float64)).to(dev) for e in host_e0]
    jq_d = torch.empty(2 * n * 2, dtype=torch.float64, device=dev)
    nf3 = m.nx * m.ny * 3
    e_d = torch.empty(2 * nf3 * 2, dtype=torch.float64, device=dev)
    h_d = torch.empty_like(e_d)
    pw = [egx.plane_wave(m, freq_to_omega(f), 0.0) for f in freqs]

    def responses(k, e, h):
        """Total fields at the surface (anomalous + plane wave) and the MT
        responses of all cell centres (Mt3DForwardSolver.cs:300-337)."""
        e_n, h_n = pw[k]
        e = e.reshape(2, nf3 // 3, 3).copy()
        h = h.reshape(2, nf3 // 3, 3).copy()
        e[0, :, 0] += e_n
        h[0, :, 1] += h_n
        e[1, :, 1] += e_n
        h[1, :, 0] -= h_n
        return egx.mt_responses(e[0], e[1], h[0], h[1], freq_to_omega(freqs[k]))
    torch.cuda.synchronize(dev)

    def step(i, where):
        """One MT solve: Green tensor, both polarisations to jQ, fields at the
        surface and the responses at every cell centre."""
        k = i % nf
        omega = freq_to_omega(freqs[k])
        g = ctx.green_build(m, omega, 10, egx.PREC_MIXED)
        try:
            if where == egx.DEVICE:
                res = ctx.solve_sources(g, None, None, m.layer_thickness, None, [0, 1], precision=egx.PREC_MIXED,
                                        mixed=mixed, where=egx.DEVICE,
                                        dev_ptrs=dict(zeta=zeta_d[k].data_ptr(), zeta0=zeta0_d[k].data_ptr(),
                                                      e0=e0_d[k].data_ptr(), jq=jq_d.data_ptr()))
                ctx.level_fields_dev(m, omega, jq_d.data_ptr(), 2, e_d.data_ptr(), h_d.data_ptr(), z=0.0,
                                     precision=egx.PREC_MIXED)
                e = e_d.cpu().numpy().view(np.complex128)
                h = h_d.cpu().numpy().view(np.complex128)
            else:
                z, z0 = host_in[k]
                jq, _, res = ctx.solve_sources(g, z, z0, m.layer_thickness, host_e0[k], [0, 1],
                                               precision=egx.PREC_MIXED, mixed=mixed)
                e, h = ctx.level_fields(m, omega, jq, z=0.0, precision=egx.PREC_MIXED)
            responses(k, e, h)
            return res
        finally:
            g.free()

    def barrier():
        torch.cuda.synchronize(dev)
        if world > 1:
            import torch.distributed as tdist
            tdist.barrier()

    for i in range(args.warmup):
        step(i, egx.DEVICE)

    # ---- timed region: inputs resident in device memory
    barrier()
    sampler = ClockSampler(local)
    sampler.start()
    # only the contraction is timed by events inside the timed region (the
    # roofline's per-launch time); the per-kernel table comes from a second,
    # profiled pass over the same steps below
    ctx.profile(True, kinds=[egx.K_CONTRACT + egx.K_C64])
    l0 = ctx.launch_count()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    results = []
    evs[0].record(stream)
    for i in range(args.steps):
        results.append(step(i, egx.DEVICE))
        evs[i + 1].record(stream)
    barrier()
    step_ms = [evs[i].elapsed_time(evs[i + 1]) for i in range(args.steps)]
    ms_total = evs[0].elapsed_time(evs[-1])
    clocks = sampler.stop()
    launches = ctx.launch_count() - l0
    kc, kms = ctx.profile_read(egx.K_CONTRACT + egx.K_C64)
    # ---- per-kernel table: the same steps again with every kind timed
    ctx.profile(True)
    for i in range(args.steps):
        step(i, egx.DEVICE)
    torch.cuda.synchronize(dev)
    kernels = {}
    for k, name in egx.KERNEL_NAMES.items():
        for off, tag in ((0, ""), (egx.K_C64, "_c64")):
            if off and k >= egx.K_C64:
                continue
            c, ms = ctx.profile_read(k + off)
            if c:
                kernels[name + tag] = {"launches": c, "ms_total": round(ms, 2), "ms_per_launch": round(ms / c, 4)}
    ctx.profile(False)

    # ---- end to end through the C ABI: host buffers in and out
    barrier()
    e0_ev, e1_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t1 = time.perf_counter()
    e0_ev.record(stream)
    for i in range(args.steps):
        step(i, egx.HOST)
    e1_ev.record(stream)
    barrier()
    ms_e2e = max(e0_ev.elapsed_time(e1_ev), (time.perf_counter() - t1) * 1e3)
    h2d = m.nx * m.ny * m.nz * 16 + m.nz * 16 + m.nz * 8 + 2 * m.nz * 16
    d2h = 2 * 2 * nf3 * 16   # E and H of both polarisations at the surface

    # ---- plain FP64 (the reference algorithm) at frequency index 1
    plain = None
    if rank == 0 and not args.no_plain and args.steps > 1 % nf:
        k = 1 % nf
        z, z0 = host_in[k]
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        g = ctx.green_build(m, freq_to_omega(freqs[k]), 10, egx.PREC_FP64)
        jq_p, _, pres = ctx.solve_sources(g, z, z0, m.layer_thickness, host_e0[k], [0, 1],
                                          precision=egx.PREC_FP64,
                                          fgmres=dict(m_out=15, m_in=10, tol=1e-6, max_restarts=100))
        g.free()
        e_p, h_p = ctx.level_fields(m, freq_to_omega(freqs[k]), jq_p, z=0.0)
        responses(k, e_p, h_p)
        p1.record(stream)
        torch.cuda.synchronize(dev)
        tplain = p0.elapsed_time(p1)
        plain = {"frequency_hz": freqs[k], "ms_per_solve": round(tplain, 1),
                 "applies_per_pol": [r["n_applies"] for r in pres],
                 "iterations": [r["iterations"] for r in pres], "true_be": [r["true_be"] for r in pres],
                 "mixed_ms_same_frequency": round(step_ms[k], 1),
                 "speedup_mixed_vs_plain": round(tplain / step_ms[k], 2)}

    ms_max, e2e_max, value = job_rate(ms_total, ms_e2e, args.steps, world, dev)

    # roofline of the contraction: algorithmic bytes per launch / event time.
    # Bytes = the stored complex64 Green blocks of the (nx+1)(ny+1) quadrant
    # read once + the spectral buffer [2nx, 2ny, 3nz] complex64 of every
    # right-hand side of the launch read and written (two with the stacked solve).
    q = (m.nx + 1) * (m.ny + 1)
    rhs = 2 if mixed["batch"] else 1
    alg_bytes = q * c64_block_entries(m.nz) * 8 + rhs * 2 * (4 * m.nx * m.ny * 3 * m.nz * 8)
    peak, peak_src = load_peaks()
    achieved = alg_bytes / (kms / kc / 1e3) / 1e9 if kc else None
    if m.nz in (16, 32, 48):
        kname = "k_contract_sb3" if rhs == 2 else "k_contract_sb"
    else:  # packed layout: the tensor-core kernel takes one source, the TMA kernel two
        kname = "k_contract_c64" if rhs == 2 else "k_contract_mma"
    roofline = {"kernel": kname, "bound": "hbm", "rhs_per_launch": rhs,
                "achieved": round(achieved, 1) if achieved else None, "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4) if achieved else None, "peak_source": peak_src,
                "algorithmic_bytes": alg_bytes, "ms_per_launch": round(kms / kc, 4) if kc else None,
                "traffic": (int(CONTRACT_TRAFFIC_BYTES[rhs]) if CONTRACT_TRAFFIC_BYTES[rhs] and (m.nx, m.ny, m.nz) == (256, 256, 48)
                            else None)}

    cpu = None
    if rank == 0 and not args.no_cpu:
        apl = int(round(np.mean(plain["applies_per_pol"]))) if plain else REFERENCE_APPLIES_PER_POL
        cpu = cpu_baseline(m, apl)

    line = {
        "metric": METRIC, "value": round(value, 5), "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64 (inner) / c128 (outer)",
        "data": "synthetic: seeded random model (5-layer background, 20 boxes), no dataset",
        "config": {"workload": "%s model %dx%dx%d, %d frequencies %.0e..%.0e Hz cycled, 2 polarisations per solve, "
                               "surface E/H and impedance/rho_a/phase at all cell centres"
                               % (args.workload, m.nx, m.ny, m.nz, nf, freqs[0], freqs[-1]),
                   "method": "mixed precision (complex64 FGMRES(30)+GMRES(10) inside FP64 refinement, tol 1e-6); "
                             + ("both polarisations as one stacked system (2-source applies); " if mixed["batch"]
                                else "polarisations solved one after the other; ")
                             + "learned preconditioner not used",
                   "green": "built in FP64 on the device inside every step",
                   "parallelism": "replicas" if world > 1 else "1 GPU",
                   "l2": "inputs larger than L2 (complex64 Green tensor 4.9 GB per frequency)"},
        "e2e": {"value": round(args.steps * world / (e2e_max / 1e3), 5), "unit": "solves/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "plain_fp64": plain,
        "clocks": clocks,
        "gpu_launches": launches,
        "launches_before_timed": l0,
        "kernels": kernels,
        "kernels_source": "a second pass over the same steps after the timed region, every kernel kind event-timed",
        "step_ms": [round(t, 1) for t in step_ms],
        "solves": [[{k: r[k] for k in ("converged", "iterations", "n_applies", "n_refinements", "true_be")}
                    for r in res] for res in results],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


# ---------------------------------------------------------------- CPU side
class CpuApply:
    """One complex128 CIE operator apply of the oracle at the model's size,
    timed on the host cores: the forward and inverse 2-D FFTs of the full
    [2nx, 2ny, 3nz] buffer (scipy.fft, all cores; FFTW's role in the
    reference) plus the threaded C block contraction (oracle/contract.c, the
    reference's per-point zspmv/zgemv) of `sample_points` spectral points --
    a sample larger than the caches -- scaled to all 4 nx ny points."""

    def __init__(self, m, sample_points=16384, seed=0):
        from oracle import ccontract
        self.cc = ccontract
        rng = np.random.default_rng(seed)
        self.m = m
        nx, ny, nz = m.nx, m.ny, m.nz
        self.cores = ccontract.max_threads()
        self.sample = sample_points
        self.buf = (rng.standard_normal((2 * nx, 2 * ny, 3 * nz))
                    + 1j * rng.standard_normal((2 * nx, 2 * ny, 3 * nz)))
        s = nz * (nz + 1) // 2
        self.G = {c: rng.standard_normal((sample_points, s)) + 1j * rng.standard_normal((sample_points, s))
                  for c in ("xx", "xy", "yy", "zz")}
        for c in ("xz", "yz"):
            self.G[c] = (rng.standard_normal((sample_points, nz * nz))
                         + 1j * rng.standard_normal((sample_points, nz * nz)))
        self.x = rng.standard_normal((sample_points, 3, nz)) + 1j * rng.standard_normal((sample_points, 3, nz))

    def seconds(self):
        import scipy.fft as sfft
        m = self.m
        t = time.perf_counter()
        spec = sfft.fft2(self.buf, axes=(0, 1), workers=self.cores)
        sfft.ifft2(spec, axes=(0, 1), workers=self.cores, overwrite_x=True)
        t_fft = time.perf_counter() - t
        del spec
        t = time.perf_counter()
        self.cc.contract(self.G, self.x, m.nz, self.cores)
        t_con = (time.perf_counter() - t) * (4 * m.nx * m.ny / self.sample)
        return t_fft + t_con, t_fft, t_con

    def describe(self, applies_per_pol, t_fft, t_con):
        m = self.m
        return ("one complex128 operator apply of the oracle: scipy 2-D FFTs of the full %dx%dx%d buffer "
                "(%.2f s) + threaded C block contraction of %d of %d spectral points, scaled (%.2f s); a solve "
                "= 2 polarisations x %d applies (the reference FGMRES count at tol 1e-6); Green build and "
                "Arnoldi not included" % (2 * m.nx, 2 * m.ny, 3 * m.nz, t_fft, self.sample, 4 * m.nx * m.ny,
                                          t_con, applies_per_pol))


def cpu_baseline(m, applies_per_pol):
    cpu = CpuApply(m)
    cpu.seconds()
    t_apply, t_fft, t_con = cpu.seconds()
    solve_s = 2 * applies_per_pol * t_apply
    return {"value": round(1.0 / solve_s, 6), "unit": "solves/s", "cores": cpu.cores, "kind": "port",
            "sample": cpu.describe(applies_per_pol, t_fft, t_con)}


def run_reference(args, rank, world):
    """Reference arm: the oracle restatement of the reference's path (the
    reference is C#/.NET, which this machine cannot run) on all host cores,
    each step a bounded sample (one operator apply) scaled to a solve."""
    if rank != 0:
        return
    m = make_model(args.workload, seed=1, mesh=args.mesh)
    cpu = CpuApply(m)
    for _ in range(args.warmup):
        cpu.seconds()
    times = []
    for _ in range(args.steps):
        t_apply, t_fft, t_con = cpu.seconds()
        times.append(2 * REFERENCE_APPLIES_PER_POL * t_apply)
    solve_s = float(np.mean(times))
    value = 1.0 / solve_s
    base = {"value": round(value, 6), "unit": "solves/s", "cores": cpu.cores, "kind": "port",
            "sample": cpu.describe(REFERENCE_APPLIES_PER_POL, t_fft, t_con)}
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 6), "unit": "solves/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(solve_s * 1e3, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic: seeded random model, no dataset",
            "config": {"workload": "%s model %dx%dx%d, 2 polarisations per solve" % (args.workload, m.nx, m.ny, m.nz),
                       "method": "reference algorithm, complex128, oracle restatement on the host cores"},
            "cpu_baseline": base,
            "e2e": {"value": round(value, 6), "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_batching(args, rank, world, local):
    """Batching configuration: 2 seeded models of uneven meshes (drawn in
    [64,192]x[64,160]x[16,40], 2N 7-smooth) x 16 frequencies over 1e-4..100 Hz,
    both polarisations per solve (64 polarisation solves), mixed precision to
    1e-6, Green tensors built inside the timed region. The stream count comes
    from the autotuner (timed on a sample, outside the timed region); the same
    batch on one stream is timed beside it."""
    import torch
    from extreme_gb300 import egx
    from extreme_gb300.batch import BatchForwardSolver, batching_models
    from extreme_gb300.forward import ForwardSettings, MixedSettings
    torch.cuda.set_device(local)
    models = batching_models(seed=7 + rank)
    freqs = list(np.logspace(-4, 2, 16))
    jobs = [(m, f) for m in models for f in freqs]
    solver = BatchForwardSolver(ForwardSettings(), precision=egx.PREC_MIXED,
                                mixed=MixedSettings(tol=1e-6, max_outer=5, m_out=30, m_in=10, inner_tol=5e-7,
                                                    inner_restarts=20), device=local)
    sampler = ClockSampler(local)
    tune = solver.tune(jobs[::4])  # 8 jobs across both models and the frequency range
    for _ in range(max(0, args.warmup - 1)):
        solver.solve(jobs[:4], streams=solver.streams)
    out = {}
    sampler.start()
    for label, n in (("tuned", solver.streams), ("one_stream", 1)):
        torch.cuda.synchronize()
        t = time.perf_counter()
        res = solver.solve(jobs, streams=n)
        torch.cuda.synchronize()
        out[label] = (time.perf_counter() - t, res)
    clocks = sampler.stop()
    dt, res = out["tuned"]
    ok = all(r["converged"] and r["true_be"] < 1e-6 for sol in res for r in sol.results)
    line = {
        "metric": "MT solves/s, batching configuration (64 polarisation solves, uneven meshes), 1 GB300",
        "value": round(len(jobs) / dt, 4), "unit": "solves/s", "n_gpus": 1, "steps": 1, "warmup": args.warmup,
        "ms_per_step": round(dt * 1e3, 1), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 (inner) / c128 (outer)", "data": "synthetic: seeded random models, no dataset",
        "config": {"workload": "batching: %s x 16 frequencies 1e-4..100 Hz x 2 polarisations"
                               % ", ".join("%dx%dx%d" % (m.nx, m.ny, m.nz) for m in models),
                   "streams": solver.streams, "tune_seconds": {str(k): round(v, 3) for k, v in tune.items()},
                   "l2": "Green tensors and buffers larger than L2"},
        "one_stream_value": round(len(jobs) / out["one_stream"][0], 4),
        "all_converged_below_1e-6": ok,
        "iterations": [[r["iterations"] for r in sol.results][0] for sol in res],
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    solver.close()


def main():
    args = parse()
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as tdist
        if args.impl == "ours":
            import torch
            torch.cuda.set_device(local)
            tdist.init_process_group("nccl")
        else:
            tdist.init_process_group("gloo")
    try:
        if args.impl == "reference":
            run_reference(args, rank, world)
        elif args.workload == "batching":
            run_batching(args, rank, world, local)
        else:
            run_ours(args, rank, world, local)
    finally:
        if world > 1:
            import torch.distributed as tdist
            tdist.destroy_process_group()


if __name__ == "__main__":
    main()
