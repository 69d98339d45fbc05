"""Benchmark: MT forward solves per second.

Default workload (``--workload precision``): the 256x256x48 precision model.
One step is one MT solve at one frequency: the Green tensor built in FP64 on
the device (stored complex64 for the inner solver and complex128 for the
refinement residual), both polarisations solved to a 1e-6 relative true
residual by the mixed-precision solve (complex64 FGMRES with a GMRES
preconditioner inside FP64 iterative refinement), then E and H at the
surface (level tensors) and the impedance, apparent resistivity and phase at
all 256x256 cell centres. Steps cycle over the model's four frequencies
(1e-3 .. 10 Hz, log-spaced).

Keys of the JSON line beyond the common ones:
  e2e          the same solves through the C ABI with page-locked host
               buffers (zeta, zeta0, dz, E0 in; jQ of both polarisations out
               and back in for the level fields; surface E and H out);
  roofline     the complex64 block-contraction kernel, its CUDA-event time on
               the library's stream during the timed region, against the
               measured HBM copy bandwidth; roofline.apply: the whole
               two-source operator apply (its five kernels) against the same;
  field_error  per frequency, the mixed step's jQ, surface E and H and
               off-diagonal apparent resistivity and phase against a
               complex128 solve of the reference algorithm to 1e-8;
  plain_fp64   one solve of the reference algorithm (complex128 FGMRES with
               the reference's defaults, tol 1e-6) at the second frequency,
               beside the timed mixed step at that frequency;
  cpu_baseline the oracle port on this host's cores: one complete
               complex128 operator apply over every spectral point on the
               device-built tensor (reference layout) and one Gram-Schmidt
               pass, scaled by this run's measured apply count of the plain
               solve (a derived rate; the sample is stated).

``--workload small`` / ``medium``: the plain configurations as configured
(complex128 FGMRES(20)+GMRES(10) to 1e-8, the configuration's frequencies,
both polarisations, surface fields and responses); the line adds
operator-applies/s and the FP64 roofline of the apply.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload precision|medium|small|batching]

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

# The learned flexible preconditioner was trained and measured on held-out
# models (2,000 seeded 128x128x32 solves) and does not gain there, so the
# timed method is the mixed form without it; the label says so.
METRIC = ("MT solves/s to 1e-6 residual (256x256x48): mixed (learned preconditioner measured, no held-out gain, "
          "not used) vs plain FP64, 1 GB300")
LEARNED_RESULT = ("trained on 2,000 seeded 128x128x32 solves (held-out loss 0.68); as the flexible preconditioner "
                  "it misses its 4-cycle budget on held-out models and falls back: 247 applies against 123 for the "
                  "GMRES(10) preconditioner at 0.01 Hz (profiles/learned_preconditioner_128x128x32.md)")
METRIC_PLAIN = "MT solves/s, plain complex128 method (FGMRES(20)+GMRES(10), tol 1e-8), %s, 1 GB300"

# DRAM bytes (read + write) of one launch of the complex64 contraction at
# 256x256x48, by right-hand sides per launch, measured by ncu at 128x128x48
# (16,641 stored points) and scaled by the stored bytes, which grow with the
# stored points. One: 1.4262 GB x 5.6765 / 1.4290; two (k_contract_ws):
# 1.5739 GB x 6.2805 / 1.5800.
CONTRACT_TRAFFIC_BYTES = {1: 5.665e9, 2: 6.256e9}

# Operator applications and outer iterations per polarisation of the plain
# reference algorithm on the seed-1 model at each of its frequencies,
# measured on one GB300 by `python bench.py --record-counts --workload W`
# into profiles/plain_fp64_counts_<mesh>.json (the file records the
# command). The reference arm, which runs no GPU code, turns its timed
# sample into a solve rate with them; the default arm re-measures the count
# at one frequency and reports whether it still matches.
def counts_file(m):
    return os.path.join(ROOT, "profiles", "plain_fp64_counts_%dx%dx%d.json" % (m.nx, m.ny, m.nz))


def counts_method(workload):
    """(FGMRES parameters, label) of the plain solve whose counts are
    recorded: the reference's defaults at the mixed form's 1e-6 for the
    precision workload, the configured FGMRES(20) at 1e-8 otherwise."""
    if workload == "precision":
        return dict(m_out=15, m_in=10, tol=1e-6, max_restarts=100), \
            "complex128 FGMRES(15) + GMRES(10), tol 1e-6 (the reference's defaults)"
    return dict(m_out=20, m_in=10, tol=1e-8, max_restarts=100), "complex128 FGMRES(20) + GMRES(10), tol 1e-8"


# FP64 peak of one GB300 (nominal; the measured peaks file covers HBM and
# bf16 only): the bound of the plain complex128 apply.
FP64_PEAK_GFLOPS_NOMINAL = 1250.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=4)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="precision", choices=["precision", "medium", "small", "batching"],
                   help="batching: the 64-solve configuration of uneven meshes")
    p.add_argument("--mesh", default=None, help="NXxNYxNZ: the same generator at another mesh (profiling cases)")
    p.add_argument("--no-plain", action="store_true", help="skip the plain FP64 solve")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    p.add_argument("--no-field-error", action="store_true", help="skip the complex128 reference solves")
    p.add_argument("--no-batch", action="store_true",
                   help="solve the two polarisations one after the other instead of as one stacked system")
    p.add_argument("--record-counts", action="store_true",
                   help="measure the plain FP64 solve's counts at every frequency and write them under profiles/")
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


def block_entries(nz):
    """Bs: algorithmic complex entries of one spectral point's Green block
    (4 packed symmetric components + 2 full ones)."""
    return 4 * (nz * (nz + 1) // 2) + 2 * nz * nz


def apply_bytes(m, s, nrhs, quadrant=True):
    """Algorithmic bytes of one operator apply of nrhs sources sharing G:
    s [Q Bs + nrhs (7 + 48) Nx Ny Nz] (G read once; x, r read and y written;
    the spectral buffer written and read on each side of the contraction);
    Q = (Nx+1)(Ny+1) stored points (quadrant) or P = 4 Nx Ny."""
    q = (m.nx + 1) * (m.ny + 1) if quadrant else 4 * m.nx * m.ny
    return s * (q * block_entries(m.nz) + nrhs * 55 * m.nx * m.ny * m.nz)


def apply_flops(m, nrhs):
    """8 * 9 Nz^2 P (contraction) + 2 * 3 Nz * 5 P log2 P (two FFTs), per source."""
    P = 4 * m.nx * m.ny
    return nrhs * (8 * 9 * m.nz ** 2 * P + 2 * 3 * m.nz * 5 * P * np.log2(P))


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


def offdiag(a):
    a = np.asarray(a).reshape(-1, 2, 2)
    return np.stack([a[:, 0, 1], a[:, 1, 0]])


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


def kernel_table(ctx, egx):
    kernels = {}
    for k, name in egx.KERNEL_NAMES.items():
        for off, tag in ((0, ""), (egx.K_C64, "_c64")):
            if off and k >= egx.K_C64:
                continue
            c, ms = ctx.profile_read(k + off)
            if c:
                kernels[name + tag] = {"launches": c, "ms_total": round(ms, 2), "ms_per_launch": round(ms / c, 4)}
    return kernels


def fields_and_responses(pw_k, omega, e, h, nf3):
    """Total surface fields (anomalous + plane wave) of both polarisations
    and the MT responses at every cell centre (Mt3DForwardSolver.cs:300-337)."""
    from extreme_gb300 import egx
    e_n, h_n = pw_k
    e = e.reshape(2, nf3 // 3, 3).copy()
    h = h.reshape(2, nf3 // 3, 3).copy()
    e[0, :, 0] += e_n
    h[0, :, 1] += h_n
    e[1, :, 1] += e_n
    h[1, :, 0] -= h_n
    z, rho, ph = egx.mt_responses(e[0], e[1], h[0], h[1], omega)
    return e, h, rho, ph


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
    zr_d = torch.empty(nf3 // 3 * 4 * 2, dtype=torch.float64, device=dev)
    rho_d = torch.empty(nf3 // 3 * 4, dtype=torch.float64, device=dev)
    ph_d = torch.empty_like(rho_d)
    pw = [egx.plane_wave(m, freq_to_omega(f), 0.0) for f in freqs]

    # page-locked host buffers of the end-to-end steps: the inputs as a caller
    # holds them, jQ and the surface fields written in place by the library
    def pinned(shape):
        return torch.empty(shape, dtype=torch.complex128, pin_memory=True).numpy()

    pin_in, pin_e0 = [], []
    for (z, z0), e in zip(host_in, host_e0):
        pz, pz0, pe = pinned(z.shape), pinned(z0.shape), pinned(e.shape)
        pz[...], pz0[...], pe[...] = z, z0, e
        pin_in.append((pz, pz0))
        pin_e0.append(pe)
    pin_jq = pinned((2, n))
    pin_eh = (pinned((2, m.nx, m.ny, 3)), pinned((2, m.nx, m.ny, 3)))
    torch.cuda.synchronize(dev)

    def step(i, where, keep=None):
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
                # the responses at every cell centre on the device; the step's
                # result read back is impedance, apparent resistivity and phase
                ctx.mt_responses_dev(e_d.data_ptr(), h_d.data_ptr(), nf3 // 3, omega, pw[k][0], pw[k][1],
                                     zr_d.data_ptr(), rho_d.data_ptr(), ph_d.data_ptr())
                rho = rho_d.cpu().numpy().reshape(-1, 2, 2)
                ph = ph_d.cpu().numpy().reshape(-1, 2, 2)
                if keep is not None:
                    e_t, h_t, _, _ = fields_and_responses(pw[k], omega, e_d.cpu().numpy().view(np.complex128),
                                                          h_d.cpu().numpy().view(np.complex128), nf3)
                    keep[k] = (jq_d.cpu().numpy().view(np.complex128).reshape(2, n).copy(), e_t, h_t, rho, ph)
            else:
                z, z0 = pin_in[k]
                jq, _, res = ctx.solve_sources(g, z, z0, m.layer_thickness, pin_e0[k], [0, 1],
                                               precision=egx.PREC_MIXED, mixed=mixed, out=pin_jq)
                e, h = ctx.level_fields(m, omega, jq, z=0.0, precision=egx.PREC_MIXED, out=pin_eh)
                fields_and_responses(pw[k], omega, e, h, nf3)
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
    # ---- per-kernel table: the same steps again with every kind timed; each
    # frequency's fields kept for the field-error comparison
    ctx.profile(True)
    kept = {}
    for i in range(args.steps):
        step(i, egx.DEVICE, keep=kept)
    torch.cuda.synchronize(dev)
    kernels = kernel_table(ctx, egx)
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
    # in: zeta, zeta0, dz, the two normal-field columns, and jQ of both
    # polarisations back in for the level fields; out: jQ, then E and H of
    # both polarisations at the surface
    h2d = m.nx * m.ny * m.nz * 16 + m.nz * 16 + m.nz * 8 + 2 * m.nz * 16 + 2 * n * 16
    d2h = 2 * n * 16 + 2 * 2 * nf3 * 16

    # ---- plain FP64 (the reference algorithm, its defaults, tol 1e-6) at
    # frequency index 1; its device-built complex128 tensor is kept on the
    # host (reference layout) for the CPU baseline
    plain, G_host = None, None
    if rank == 0 and not args.no_plain and args.steps > 1 % nf:
        k = 1 % nf
        z, z0 = host_in[k]
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        g = ctx.green_build(m, freq_to_omega(freqs[k]), 10, egx.PREC_FP64)
        jq_p, _, pres = ctx.solve_sources(g, z, z0, m.layer_thickness, host_e0[k], [0, 1],
                                          precision=egx.PREC_FP64,
                                          fgmres=dict(m_out=15, m_in=10, tol=1e-6, max_restarts=100))
        e_p, h_p = ctx.level_fields(m, freq_to_omega(freqs[k]), jq_p, z=0.0)
        fields_and_responses(pw[k], freq_to_omega(freqs[k]), e_p, h_p, nf3)
        p1.record(stream)
        torch.cuda.synchronize(dev)
        tplain = p0.elapsed_time(p1)
        if not args.no_cpu:
            G_host = g.download()
        g.free()
        plain = {"frequency_hz": freqs[k], "ms_per_solve": round(tplain, 1),
                 "applies_per_pol": [r["n_applies"] for r in pres],
                 "iterations": [r["iterations"] for r in pres], "true_be": [r["true_be"] for r in pres],
                 "mixed_ms_same_frequency": round(step_ms[k], 1),
                 "speedup_mixed_vs_plain": round(tplain / step_ms[k], 2)}
        rec = read_counts(m)
        if rec:
            want = [r for r in rec["per_frequency"] if abs(r["frequency_hz"] - freqs[k]) < 1e-12 * freqs[k]]
            plain["counts_match_recorded"] = bool(want) and want[0]["applies_per_pol"] == plain["applies_per_pol"]

    # ---- field error of the mixed steps against complex128 solves to 1e-8
    field = None
    if rank == 0 and not args.no_field_error:
        field = field_errors(ctx, m, freqs, host_in, host_e0, pw, kept, nf3)

    ms_max, e2e_max, value = job_rate(ms_total, ms_e2e, args.steps, world, dev)

    # roofline of the contraction: algorithmic bytes per launch / event time.
    # Bytes = the stored complex64 Green blocks of the (nx+1)(ny+1) quadrant
    # (Bs entries each, the padding of the sub-block layout not counted)
    # read once + the spectral buffer [2nx, 2ny, 3nz] complex64 of every
    # right-hand side of the launch read and written (two with the stacked solve).
    q = (m.nx + 1) * (m.ny + 1)
    rhs = 2 if mixed["batch"] else 1
    alg_bytes = q * block_entries(m.nz) * 8 + rhs * 2 * (4 * m.nx * m.ny * 3 * m.nz * 8)
    peak, peak_src = load_peaks()
    achieved = alg_bytes / (kms / kc / 1e3) / 1e9 if kc else None
    if m.nz in (16, 32, 48):
        kname = "k_contract_ws" if rhs == 2 else "k_contract_sb"
    else:  # packed layout: the tensor-core kernel takes one source, the TMA kernel two
        kname = "k_contract_c64" if rhs == 2 else "k_contract_mma"
    roofline = {"kernel": kname, "bound": "hbm", "rhs_per_launch": rhs,
                "achieved": round(achieved, 1) if achieved else None, "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4) if achieved else None, "peak_source": peak_src,
                "algorithmic_bytes": alg_bytes, "ms_per_launch": round(kms / kc, 4) if kc else None,
                "stored_bytes_per_launch": q * c64_block_entries(m.nz) * 8 + rhs * 2 * (4 * m.nx * m.ny * 3 * m.nz * 8),
                "traffic": (int(CONTRACT_TRAFFIC_BYTES[rhs]) if CONTRACT_TRAFFIC_BYTES[rhs] and (m.nx, m.ny, m.nz) == (256, 256, 48)
                            else None)}
    # the whole apply: its five kernels' mean event times per apply launch
    parts = ("fwd_y_c64", "fwd_x_c64", "contract_c64", "bwd_x_c64", "bwd_y_c64")
    if all(p in kernels for p in parts):
        per = {p: kernels[p]["ms_total"] / kernels["contract_c64"]["launches"] for p in parts}
        t_apply = sum(per.values())
        ab = apply_bytes(m, 8, rhs)
        roofline["apply"] = {"kernels": {p: round(v, 4) for p, v in per.items()}, "ms_per_apply": round(t_apply, 4),
                             "algorithmic_bytes": ab, "achieved": round(ab / (t_apply / 1e3) / 1e9, 1),
                             "frac": round(ab / (t_apply / 1e3) / 1e9 / peak, 4),
                             "reference_layout_bytes": apply_bytes(m, 8, rhs, quadrant=False)}

    cpu = None
    if rank == 0 and not args.no_cpu and plain is not None and G_host is not None:
        from extreme_gb300.model import OmegaModel
        om = OmegaModel.build(m, freqs[1 % nf])
        cpu = cpu_baseline(m, om, G_host, plain, sample_x=jq_p[0])
        del G_host

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
                   "learned": LEARNED_RESULT,
                   "green": "built in FP64 on the device inside every step",
                   "parallelism": "replicas" if world > 1 else "1 GPU",
                   "l2": "inputs larger than L2 (complex64 Green tensor 4.9 GB per frequency)"},
        "e2e": {"value": round(args.steps * world / (e2e_max / 1e3), 5), "unit": "solves/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "plain_fp64": plain,
        "field_error": field,
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


def field_errors(ctx, m, freqs, host_in, host_e0, pw, kept, nf3):
    """Per frequency: the mixed step's jQ, total surface E and H and the
    off-diagonal apparent resistivity and phase against the reference
    algorithm in complex128 (FP64 Green tensor and level tensors,
    FGMRES(20)+GMRES(10) to 1e-8), relative L2 norms over both
    polarisations and all cell centres."""
    from extreme_gb300 import egx
    from extreme_gb300.model import freq_to_omega
    n = m.nx * m.ny * 3 * m.nz
    rows = []
    for k, f in enumerate(freqs):
        if k not in kept:
            continue
        omega = freq_to_omega(f)
        z, z0 = host_in[k]
        g = ctx.green_build(m, omega, 10, egx.PREC_FP64)
        try:
            jq, _, res = ctx.solve_sources(g, z, z0, m.layer_thickness, host_e0[k], [0, 1],
                                           precision=egx.PREC_FP64,
                                           fgmres=dict(m_out=20, m_in=10, tol=1e-8, max_restarts=100))
        finally:
            g.free()
        e, h = ctx.level_fields(m, omega, jq, z=0.0)
        e, h, rho, ph = fields_and_responses(pw[k], omega, e, h, nf3)
        jq_m, e_m, h_m, rho_m, ph_m = kept[k]
        rows.append({"frequency_hz": f, "jq": rel(jq_m, jq.reshape(2, n)), "e": rel(e_m, e), "h": rel(h_m, h),
                     "rho_offdiag": rel(offdiag(rho_m), offdiag(rho)),
                     "phase_offdiag": rel(offdiag(ph_m), offdiag(ph)),
                     "reference_true_be": [r["true_be"] for r in res]})
    worst = max(max(r[c] for c in ("jq", "e", "h", "rho_offdiag", "phase_offdiag")) for r in rows) if rows else None
    return {"per_frequency": rows, "max": worst, "bar": 1e-5,
            "reference": "complex128 reference algorithm on the device (FP64 Green and level tensors, "
                         "FGMRES(20)+GMRES(10) to 1e-8), parity-tested against the oracle up to 32x32x32 "
                         "and on the 128x128x32 apply",
            "norm": "relative L2 over both polarisations and all cell centres (rho_a, phase: xy and yx)"}


# ---------------------------------------------------------------- plain configurations
def run_plain(args, rank, world, local):
    """The plain configurations as configured: complex128 FGMRES(20) with the
    GMRES(10) preconditioner to 1e-8, both polarisations, every configured
    frequency (small: 0.1 Hz; medium: 4 frequencies 1e-3..10 Hz), surface
    fields and responses at every cell centre. One step = one MT solve at one
    frequency, Green tensor (FP64) built inside the step."""
    import torch

    from extreme_gb300 import egx
    from extreme_gb300.forward import model_zeta
    from extreme_gb300.model import freq_to_omega

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    m = make_model(args.workload, seed=1 + rank, mesh=args.mesh)
    freqs = [0.1] if args.workload == "small" else list(m.frequencies)
    nf = len(freqs)
    ctx = egx.Context(local)
    stream = torch.cuda.Stream(dev)
    ctx.set_stream(stream.cuda_stream)
    ctx.level_cache(0)
    n = m.nx * m.ny * 3 * m.nz
    nf3 = m.nx * m.ny * 3
    fg = dict(m_out=20, m_in=10, tol=1e-8, max_restarts=100)
    host_in = [model_zeta(m, freq_to_omega(f)) for f in freqs]
    host_e0 = [np.ascontiguousarray(np.stack([egx.normal_field(m, freq_to_omega(f))] * 2)) for f in freqs]
    zeta_d = [torch.from_numpy(z.reshape(-1).view(np.float64)).to(dev) for z, _ in host_in]
    zeta0_d = [torch.from_numpy(z0.view(np.float64)).to(dev) for _, z0 in host_in]
    e0_d = [torch.from_numpy(e.reshape(-1).view(np.float64)).to(dev) for e in host_e0]
    jq_d = torch.empty(2 * n * 2, dtype=torch.float64, device=dev)
    e_d = torch.empty(2 * nf3 * 2, dtype=torch.float64, device=dev)
    h_d = torch.empty_like(e_d)
    zr_d = torch.empty(nf3 // 3 * 4 * 2, dtype=torch.float64, device=dev)
    rho_d = torch.empty(nf3 // 3 * 4, dtype=torch.float64, device=dev)
    ph_d = torch.empty_like(rho_d)
    pw = [egx.plane_wave(m, freq_to_omega(f), 0.0) for f in freqs]

    def step(i, where):
        k = i % nf
        omega = freq_to_omega(freqs[k])
        g = ctx.green_build(m, omega, 10, egx.PREC_FP64)
        try:
            if where == egx.DEVICE:
                res = ctx.solve_sources(g, None, None, m.layer_thickness, None, [0, 1], precision=egx.PREC_FP64,
                                        fgmres=fg, where=egx.DEVICE,
                                        dev_ptrs=dict(zeta=zeta_d[k].data_ptr(), zeta0=zeta0_d[k].data_ptr(),
                                                      e0=e0_d[k].data_ptr(), jq=jq_d.data_ptr()))
                ctx.level_fields_dev(m, omega, jq_d.data_ptr(), 2, e_d.data_ptr(), h_d.data_ptr(), z=0.0)
                e = e_d.cpu().numpy().view(np.complex128)
                h = h_d.cpu().numpy().view(np.complex128)
            else:
                z, z0 = host_in[k]
                jq, _, res = ctx.solve_sources(g, z, z0, m.layer_thickness, host_e0[k], [0, 1],
                                               precision=egx.PREC_FP64, fgmres=fg)
                e, h = ctx.level_fields(m, omega, jq, z=0.0)
            fields_and_responses(pw[k], omega, e, h, nf3)
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
    barrier()
    sampler = ClockSampler(local)
    sampler.start()
    ctx.profile(True, kinds=[egx.K_CONTRACT])
    l0 = ctx.launch_count()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    results = []
    ev[0].record(stream)
    for i in range(args.steps):
        results.append(step(i, egx.DEVICE))
    ev[1].record(stream)
    barrier()
    ms_total = ev[0].elapsed_time(ev[1])
    clocks = sampler.stop()
    launches = ctx.launch_count() - l0
    kc, kms = ctx.profile_read(egx.K_CONTRACT)
    ctx.profile(True)
    for i in range(args.steps):
        step(i, egx.DEVICE)
    torch.cuda.synchronize(dev)
    kernels = kernel_table(ctx, egx)
    ctx.profile(False)
    barrier()
    t1 = time.perf_counter()
    for i in range(args.steps):
        step(i, egx.HOST)
    barrier()
    ms_e2e = (time.perf_counter() - t1) * 1e3
    ms_max, e2e_max, value = job_rate(ms_total, ms_e2e, args.steps, world, dev)
    applies = sum(r["n_applies"] for res in results for r in res)
    peak, peak_src = load_peaks()
    parts = ("fwd_y", "fwd_x", "contract", "bwd_x", "bwd_y")
    roof = None
    if all(p in kernels for p in parts):
        nl = kernels["contract"]["launches"]
        t_apply = sum(kernels[p]["ms_total"] for p in parts) / nl
        ab = apply_bytes(m, 16, 1)
        fl = apply_flops(m, 1)
        roof = {"kernel": "operator apply (fwd_y, fwd_x, contract, bwd_x, bwd_y), complex128, one source",
                "ms_per_apply": round(t_apply, 4), "algorithmic_bytes": ab, "flops": fl,
                "hbm_frac": round(ab / (t_apply / 1e3) / 1e9 / peak, 4),
                "fp64_frac": round(fl / (t_apply / 1e3) / 1e9 / FP64_PEAK_GFLOPS_NOMINAL, 4),
                "peak_hbm_gbs": peak, "peak_hbm_source": peak_src,
                "peak_fp64_gflops": FP64_PEAK_GFLOPS_NOMINAL, "peak_fp64_source": "nominal",
                "bound": "fp64" if fl / FP64_PEAK_GFLOPS_NOMINAL > ab / peak else "hbm",
                "contract_ms_per_launch": round(kms / kc, 4) if kc else None}
    line = {
        "metric": METRIC_PLAIN % ("%dx%dx%d" % (m.nx, m.ny, m.nz)), "value": round(value, 5), "unit": "solves/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": "synthetic: seeded model of the configuration, no dataset",
        "config": {"workload": "%s model %dx%dx%d, frequencies %s Hz, 2 polarisations per solve, surface E/H and "
                               "responses at all cell centres" % (args.workload, m.nx, m.ny, m.nz,
                                                                  ", ".join("%g" % f for f in freqs)),
                   "method": "reference algorithm in complex128: FGMRES(20) + GMRES(10) preconditioner, tol 1e-8",
                   "green": "built in FP64 on the device inside every step",
                   "l2": "flushed by the Green build of every step (%s)" % (
                       "tensor and buffers larger than L2" if args.workload == "medium" else
                       "the small model's working set fits in L2")},
        "operator_applies_per_s": round(applies * world / (ms_max / 1e3), 2),
        "applies_per_solve": round(applies / args.steps, 1),
        "e2e": {"value": round(args.steps * world / (e2e_max / 1e3), 5), "unit": "solves/s",
                "h2d_bytes_per_step": m.nx * m.ny * m.nz * 16 + m.nz * 16 + m.nz * 8 + 2 * m.nz * 16,
                "d2h_bytes_per_step": 2 * 2 * nf3 * 16},
        "roofline": roof, "clocks": clocks, "gpu_launches": launches, "kernels": kernels,
        "solves": [[{k: r[k] for k in ("converged", "iterations", "n_applies", "true_be")} for r in res]
                   for res in results],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


def record_counts(args):
    """Plain FP64 solves (the reference's defaults, tol 1e-6) of both
    polarisations at every frequency of the model: the counts the reference
    arm scales its timed sample by."""
    import torch

    from extreme_gb300 import egx
    from extreme_gb300.forward import model_zeta
    from extreme_gb300.model import freq_to_omega
    torch.cuda.set_device(0)
    m = make_model(args.workload, seed=1, mesh=args.mesh)
    fg, label = counts_method(args.workload)
    ctx = egx.Context(0)
    rows = []
    for f in ([0.1] if args.workload == "small" else m.frequencies):
        omega = freq_to_omega(f)
        z, z0 = model_zeta(m, omega)
        e0 = np.stack([egx.normal_field(m, omega)] * 2)
        g = ctx.green_build(m, omega, 10, egx.PREC_FP64)
        t = time.perf_counter()
        _, _, res = ctx.solve_sources(g, z, z0, m.layer_thickness, e0, [0, 1], precision=egx.PREC_FP64,
                                      fgmres=fg)
        dt = time.perf_counter() - t
        g.free()
        rows.append({"frequency_hz": f, "applies_per_pol": [r["n_applies"] for r in res],
                     "iterations": [r["iterations"] for r in res], "true_be": [r["true_be"] for r in res],
                     "gpu_solve_s": round(dt, 2)})
    ctx.close()
    out = {"command": "python bench.py --record-counts --workload %s" % args.workload
                      + (" --mesh %s" % args.mesh if args.mesh else ""),
           "model": "seed 1, %s generator" % args.workload, "mesh": [m.nx, m.ny, m.nz],
           "method": label, "per_frequency": rows}
    with open(counts_file(m), "w") as fh:
        json.dump(out, fh, indent=1)
    print(json.dumps(out))


def read_counts(m):
    try:
        with open(counts_file(m)) as fh:
            rec = json.load(fh)
    except (OSError, ValueError):
        return None
    return rec if tuple(rec.get("mesh", ())) == (m.nx, m.ny, m.nz) else None


# ---------------------------------------------------------------- CPU side
class CpuSample:
    """The oracle port of one solve's repeated work on the host cores: one
    complete complex128 operator apply over every spectral point (scipy 2-D
    FFTs and the threaded C block contraction, ``oracle/cpu_apply.py``)
    reading a Green tensor in the reference's layout (all 4 nx ny points
    stored), and one classical Gram-Schmidt pass at basis size j + 1 on
    N-vectors (``Gmres.cs:297-313``)."""

    def __init__(self, m, om, G, x, threads=0, j=5):
        from oracle import ccontract, cpu_apply
        from oracle import operator as op
        self.m = m
        self.threads = threads or ccontract.max_threads()
        self.op = cpu_apply.ThreadedOperator(G, om, op.OP_A, self.threads)
        self.x = np.ascontiguousarray(x, np.complex128).reshape(-1)
        self.j = j
        rng = np.random.default_rng(0)
        n = self.x.size
        V = np.empty((n, j + 1), np.complex128)
        for c in range(j + 1):   # an orthonormal-sized basis: unit columns
            v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
            V[:, c] = v / np.linalg.norm(v)
        self.V = V
        self.icgs = cpu_apply.icgs_pass

    def time_apply(self, threads=None):
        if threads is not None:
            self.op.threads = threads
        t = time.perf_counter()
        self.op(self.x)
        dt = time.perf_counter() - t
        self.op.threads = self.threads
        return dt

    def time_icgs(self):
        w = self.x.copy()
        t = time.perf_counter()
        self.icgs(self.V, self.j, w)
        return time.perf_counter() - t


def cpu_baseline(m, om, G, plain, sample_x):
    """The timed sample (after one untimed apply): one all-core apply, one
    Gram-Schmidt pass, one single-thread apply; the solve time is derived as
    sum over both polarisations of applies x (apply + pass), with this run's
    measured apply counts of the plain solve."""
    s = CpuSample(m, om, G, sample_x)
    s.time_apply()
    t_apply = s.time_apply()
    t_icgs = s.time_icgs()
    t_apply_1 = s.time_apply(threads=1)
    applies = sum(plain["applies_per_pol"])
    solve_s = applies * (t_apply + t_icgs)
    solve_s_1 = applies * (t_apply_1 + t_icgs)
    return {"value": round(1.0 / solve_s, 6), "unit": "solves/s", "cores": s.threads, "kind": "port",
            "derived": True,
            "sample": ("timed: one complete complex128 operator apply of the oracle port over all %d spectral "
                       "points (scipy FFTs of the %dx%dx%d buffer + threaded C block contraction on the device-"
                       "built Green tensor in the reference layout, %.1f GB) = %.3f s, and one Gram-Schmidt pass "
                       "at j = %d on N = %d = %.3f s; derived: %d applies (both polarisations, this run's plain "
                       "FP64 solve at %.3g Hz) x (apply + pass); Green build and Givens work not included"
                       % (4 * m.nx * m.ny, 2 * m.nx, 2 * m.ny, 3 * m.nz,
                          sum(v.nbytes for v in G.values()) / 1e9, t_apply, s.j, s.x.size, t_icgs, applies,
                          plain["frequency_hz"])),
            "apply_s": round(t_apply, 4), "icgs_pass_s": round(t_icgs, 4),
            "single_thread": {"apply_s": round(t_apply_1, 3), "value": round(1.0 / solve_s_1, 7), "cores": 1}}


def reference_green(m, frequency, n_src=16):
    """A Green tensor of the reference layout at the model's full spectral
    size for the reference arm: the oracle's tensor of the same layered model
    and frequency on an n_src x n_src lateral grid, tiled over the
    [2nx, 2ny] spectral grid. The reference arm runs no device code, and the
    oracle's build of the full-size tensor takes hours on the host; the
    contraction's time does not depend on the values (complex128 FMAs on
    normal numbers): the default arm times the same apply on the
    device-built tensor (its cpu_baseline.apply_s)."""
    import copy

    from extreme_gb300.model import OmegaModel
    from oracle import green
    ms = copy.deepcopy(m)
    ms.nx, ms.ny = min(n_src, m.nx), min(n_src, m.ny)
    ms.sigma = np.ascontiguousarray(m.sigma[:ms.nx, :ms.ny])
    small = green.green_tensor(OmegaModel.build(ms, frequency), 10)
    out = {}
    for c, v in small.items():
        reps = (-(-2 * m.nx // v.shape[0]), -(-2 * m.ny // v.shape[1]), 1)
        out[c] = np.ascontiguousarray(np.tile(v, reps)[:2 * m.nx, :2 * m.ny])
    return out


def run_reference(args, rank, world):
    """Reference arm: the oracle port of the reference's path (the reference
    is C#/.NET, which no machine here can run) on all host cores. Each step
    is a bounded sample of one solve's repeated work -- one complete
    complex128 operator apply over every spectral point and one Gram-Schmidt
    pass -- and ms_per_step is its measured time; the solves/s `value` is
    derived from it with the recorded apply count of the plain FP64 solve."""
    if rank != 0:
        return
    if args.workload == "small" and not args.mesh:
        return run_reference_small(args, world)
    from extreme_gb300.model import OmegaModel
    m = make_model(args.workload, seed=1, mesh=args.mesh)
    freqs = list(m.frequencies) if args.workload != "small" else [0.1]
    rec = read_counts(m)
    counts = [sum(r["applies_per_pol"]) for r in rec["per_frequency"]] if rec else None
    k = 1 % len(freqs)
    om = OmegaModel.build(m, freqs[k])
    t0 = time.perf_counter()
    G = reference_green(m, freqs[k])
    t_green_setup = time.perf_counter() - t0
    rng = np.random.default_rng(3)
    x = rng.standard_normal(m.nx * m.ny * 3 * m.nz) + 1j * rng.standard_normal(m.nx * m.ny * 3 * m.nz)
    s = CpuSample(m, om, G, x)
    for _ in range(args.warmup):
        s.time_apply()
        s.time_icgs()
    times, ta, ti = [], [], []
    for _ in range(args.steps):
        t = time.perf_counter()
        a = s.time_apply()
        i = s.time_icgs()
        times.append(time.perf_counter() - t)
        ta.append(a)
        ti.append(i)
    t_apply_1 = s.time_apply(threads=1)
    step_s = float(np.mean(times))
    applies = float(np.mean(counts)) if counts else None
    solve_s = applies * step_s if applies else None
    value = 1.0 / solve_s if solve_s else None
    sample = ("each step: one complete complex128 operator apply of the oracle port over all %d spectral points "
              "(scipy 2-D FFTs of the %dx%dx%d buffer on %d threads + threaded C block contraction, Green tensor "
              "in the reference layout, %.1f GB: the oracle's tensor of the same layered model on a 16x16 "
              "lateral grid tiled over the spectral grid) and one Gram-Schmidt pass at j = %d; value derived: "
              "mean over the frequencies of the recorded applies per solve (both polarisations, %s) x "
              "measured step time; Green build not included"
              % (4 * m.nx * m.ny, 2 * m.nx, 2 * m.ny, 3 * m.nz, s.threads,
                 sum(v.nbytes for v in G.values()) / 1e9, s.j,
                 os.path.relpath(counts_file(m), ROOT) if counts else "counts missing"))
    base = {"value": round(value, 6) if value else None, "unit": "solves/s", "cores": s.threads, "kind": "port",
            "derived": True, "sample": sample}
    # the precision workload's arm matches the headline metric; the medium
    # workload's matches the plain complex128 configuration our arm runs
    metric = METRIC if args.workload == "precision" or args.mesh else METRIC_PLAIN % ("%dx%dx%d" % (m.nx, m.ny, m.nz))
    line = {"impl": "reference", "metric": metric, "value": round(value, 6) if value else None, "unit": "solves/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_s * 1e3, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic: seeded random model, no dataset",
            "config": {"workload": "%s model %dx%dx%d, 2 polarisations per solve" % (args.workload, m.nx, m.ny,
                                                                                  m.nz),
                       "method": "reference algorithm, complex128, oracle port on the host cores"},
            "cpu_baseline": base,
            "derived_from": {"applies_per_solve": applies, "step_s": round(step_s, 4),
                             "apply_s": round(float(np.mean(ta)), 4), "icgs_pass_s": round(float(np.mean(ti)), 4),
                             "single_thread_apply_s": round(t_apply_1, 3),
                             "single_thread_value": round(1.0 / (applies * (t_apply_1 + np.mean(ti))), 7)
                             if applies else None,
                             "green_setup_s": round(t_green_setup, 1)},
            "e2e": {"value": round(value, 6) if value else None, "unit": "solves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_reference_small(args, world):
    """Reference arm of the small configuration, measured whole: every step
    is one complete MT solve of the oracle port at 0.1 Hz -- the FP64 Green
    tensor, both polarisations to 1e-8 (FGMRES(20)+GMRES(10)), the surface
    fields and the responses at every cell centre (numpy/scipy, one
    process)."""
    from extreme_gb300.model import OmegaModel
    from oracle import atoo, ccontract, cpu_apply, green, mt
    m = make_model("small", seed=1)
    om = OmegaModel.build(m, 0.1)
    threads = ccontract.max_threads()

    def solve():
        G = green.green_tensor(om, 10)
        outs = {p: mt.solve_polarization(om, G, p, m_out=20, m_in=10, tol=1e-8,
                                         make_op=lambda G_, om_, t: cpu_apply.ThreadedOperator(G_, om_, t, threads))
                for p in "xy"}
        atoo.level_responses(om, atoo.Level(0.0, 0.0, 0.0), outs["x"].jq, outs["y"].jq)
        return outs
    for _ in range(min(args.warmup, 1)):
        solve()
    t = time.perf_counter()
    for _ in range(args.steps):
        outs = solve()
    step_s = (time.perf_counter() - t) / args.steps
    value = 1.0 / step_s
    sample = ("each step one complete MT solve of the oracle port: FP64 Green tensor (numpy), both polarisations "
              "to 1e-8 (%d and %d outer iterations; operator applies on %d threads: scipy FFTs + threaded C "
              "contraction), surface fields and responses (numpy); warm-up capped at one step"
              % (outs["x"].result.iterations, outs["y"].result.iterations, threads))
    line = {"impl": "reference", "metric": METRIC_PLAIN % "32x32x8", "value": round(value, 5), "unit": "solves/s",
            "n_gpus": world, "steps": args.steps, "warmup": min(args.warmup, 1),
            "ms_per_step": round(step_s * 1e3, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic: the small configuration's model",
            "config": {"workload": "small model 32x32x8, 0.1 Hz, 2 polarisations per solve",
                       "method": "reference algorithm, complex128, oracle port on the host"},
            "cpu_baseline": {"value": round(value, 5), "unit": "solves/s", "cores": threads, "kind": "port",
                             "derived": False, "sample": sample},
            "e2e": {"value": round(value, 5), "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_batching(args, rank, world, local):
    """Batching configuration: 2 seeded models of uneven meshes (drawn in
    [64,192]x[64,160]x[16,40], 2N 7-smooth) x 16 frequencies over 1e-4..100 Hz,
    both polarisations per solve (64 polarisation solves), mixed precision to
    1e-6, Green tensors built inside the timed region. The autotuner (outside
    the timed region) picks the apply's kernel variants per mesh and the
    (stream count, CUDA-graph inner cycles) pair; the same batch on one stream
    with launched inner cycles and the built-in kernel variants is timed
    beside it."""
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
    variants, apply_times = dict(solver.variants), dict(solver.apply_times)
    for _ in range(max(0, args.warmup - 1)):
        solver.solve(jobs[:4], streams=solver.streams)
    out = {}
    sampler.start()
    torch.cuda.synchronize()
    t = time.perf_counter()
    res = solver.solve(jobs, streams=solver.streams, graphs=solver.graphs)
    torch.cuda.synchronize()
    out["tuned"] = (time.perf_counter() - t, res)
    # the baseline: one stream, launched inner cycles, built-in kernel variants
    solver.variants = {}
    torch.cuda.synchronize()
    t = time.perf_counter()
    base = solver.solve(jobs, streams=1, graphs=False)
    torch.cuda.synchronize()
    out["one_stream"] = (time.perf_counter() - t, base)
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
                   "streams": solver.streams, "graphs": solver.graphs,
                   "tune_seconds": {"%d streams, graphs %s" % k: round(v, 3) for k, v in tune.items()},
                   "apply_variants": {"%dx%dx%d" % k: {"fft_tile": v[0], "contract_variant": v[1],
                                                       "ms_per_apply": {"%d/%d" % tv: round(ms, 4)
                                                                        for tv, ms in apply_times[k].items()}}
                                      for k, v in variants.items()},
                   "l2": "Green tensors and buffers larger than L2"},
        "one_stream_value": round(len(jobs) / out["one_stream"][0], 4),
        "one_stream_method": "1 stream, launched inner cycles, built-in kernel variants",
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
    if args.record_counts:
        record_counts(args)
        return
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
        elif args.workload in ("small", "medium"):
            run_plain(args, rank, world, local)
        else:
            run_ours(args, rank, world, local)
    finally:
        if world > 1:
            import torch.distributed as tdist
            tdist.destroy_process_group()


if __name__ == "__main__":
    main()
