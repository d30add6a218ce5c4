"""Throughput benchmark of the lattice hot path (one JSON line on rank 0).

Metric: site-updates/s at 512^3 -- one site-update is one full leapfrog step
(kick + drift) of the complex field phi and all six u_ij at one lattice site.
The headline arm is the FP32-mixed fused path (FP32 fields and stencil,
Kahan-compensated drifts, FP64 host scalars); the FP64-plain drop-in path
(reference-structured separate kick and drift passes) is measured in the same
run and reported beside it.

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]

--impl reference times the reference algorithm on the host cores: the CPU
restatement of evolve.f90 (the reference Fortran/MPI/MKL build cannot be
compiled in this environment), FP64, all host threads, same lattice.
Multi-GPU: the path runs as independent replicas (one lattice per rank, no
data-path collective); value is the aggregate over ranks (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "site-updates/s at 512³ (FP32-mixed vs FP64 plain, 1 GB300); % HBM roofline"
UNIT = "site-updates/s"
# algorithmic HBM bytes per site-update (state read once + written once):
#   FP32-mixed fused Mode U: read phi 8 + phi' 8 + c_phi 8 + u 24 + u' 24 + c_u 24, write the same
#   FP64-plain Mode U:       drift 192 + kick 192 (phi 16, phi' 16, u 48, u' 48 read; 16 + 48 written each)
BYTES_PER_SITE = {"fused_kd_fp32_uij": 192, "fused_kd_fp32_phi": 48, "fused_kd_fp64_uij": 256,
                  "fused_kd_fp64_phi": 64, "kick_fp64_plain": 192, "drift_fp64": 192}
BYTES_PER_SITE_PHI_ONLY = {"kick_fp64_plain": 48, "drift_fp64": 48}


def env_rank():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def replica_time_ms(ms: float, dist) -> float:
    """The job's time is the slowest replica's: max over ranks of the timed
    region (NCCL on the GPU, gloo on host tensors)."""
    if dist is None:
        return ms
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world: int, sites: float, steps: int, ms: float) -> float:
    """Whole-job site-updates/s: every replica advances its own lattice."""
    return world * sites * steps / (ms * 1e-3)


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic_per_site(kernel: str):
    """DRAM bytes per site of `kernel` from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", f"{kernel}.md")
    try:
        txt = open(path).read()
    except OSError:
        return None
    m = re.search(r"dram_bytes_per_site:\s*([0-9.eE+-]+)", txt)
    return float(m.group(1)) if m else None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def mark(self, which: str):
        setattr(self, which, time.time())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        """Samples received while the timed region ran (host arrival time;
        nvidia-smi output is line buffered at 50 ms)."""
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        t0 = getattr(self, "start", 0.0)
        t1 = getattr(self, "stop", float("inf")) + 0.06
        for tr, ln in self.lines:
            if not (t0 <= tr <= t1):
                continue
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 10:
                continue
            try:
                sm.append(float(parts[2]))
                mx.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[6:10]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


WORKLOAD_KW = dict(potential=0, sigma_cr=1.0, kappa=0.1, seed=1)  # potential 0: potential.f90


def workload_params(ag, n, precision, gw, device=0):
    # 512^3 periodic lattice, reference potential (potential.f90), sigma_cr = 1,
    # dx = boxsize * tau_fin / N with boxsize 1, tau_fin 32; kappa 0.1.
    return ag.default_params(ngrid=n, precision=precision, gw_mode=gw, dspa=32.0 / n, device=device, **WORKLOAD_KW)


def workload_name(n):
    """config.workload of both arms: the work one step does, independent of
    the implementation that does it."""
    return (f"{n}^3 periodic lattice, one leapfrog step (kick+drift) of phi and six u_ij per site "
            f"(one site-update = one kick+drift of all 7 fields at one site); reference potential "
            f"(potential.f90), Gaussian-flat seeded IC (Philox key 1, |k| <= 2 pi / (8 dx))")


def bench_ours(ag, n, precision, gw, steps, warmup, dist, device, t0=2.0, eps=0.25, clocks=False,
               tune=True, tile=None):
    p = workload_params(ag, n, precision, gw, device)
    lat = ag.Lattice(p)
    try:
        lat.ic_gaussian_flat(kcut=2.0 * np.pi / (8 * p.dspa))
        dt, _ = lat.get_dtau(t0, 32.0, eps)
        if tile is not None and precision != ag.PREC_FP64_PLAIN:
            lat.set_tile(tile)
        elif tune and precision != ag.PREC_FP64_PLAIN:
            try:
                tile, _ = lat.autotune(3)
            except ag.AxgError:
                # the tuner snapshots the state; without room for it the
                # library's default shape runs
                tile = None
        else:
            tile = None
        t = t0
        lat.leapfrog(t, dt, 1, True, False)  # half drift + one step
        t += dt * 1.5
        lat.leapfrog(t, dt, warmup, False, False)
        t += dt * warmup
        lat.synchronize()
        lat.set_kernel_timing(True)
        if dist is not None:
            dist.barrier()
        lat.synchronize()
        sampler = ClockSampler(device) if clocks else None
        if sampler:
            sampler.__enter__()
            time.sleep(0.5)  # let nvidia-smi start streaming before the timed region
            sampler.mark("start")
        l0 = lat.launch_count()
        lat.event_record(0)
        lat.leapfrog(t, dt, steps, False, False)
        lat.event_record(1)
        ms = lat.event_elapsed(0, 1)
        lat.synchronize()
        l1 = lat.launch_count()
        if sampler:
            sampler.mark("stop")
            time.sleep(0.1)
            sampler.__exit__(None, None, None)
        if dist is not None:
            dist.barrier()
        kt = lat.kernel_timings()
        lat.set_kernel_timing(False)
        return {"ms": ms, "launches": l1 - l0, "kernels": kt, "tile": tile,
                "tile_shape": lat.tiles()[tile] if tile is not None else None,
                "clocks": sampler.summary() if sampler else None, "dt": dt, "lat": lat, "t": t + dt * steps}
    except Exception:
        lat.close()
        raise


def bench_e2e(ag, lat, n, nsub, reps, t, dt):
    """Through the public C-ABI with host buffers: per interval upload phi and
    phidot (complex128, pinned host memory), nsub leapfrog steps, download
    phi and phidot -- the host-resident data1/data2 of the reference."""
    import torch

    shape = (n, n, n, 2)
    h_phi = torch.empty(shape, dtype=torch.float64, pin_memory=True)
    h_phid = torch.empty(shape, dtype=torch.float64, pin_memory=True)
    lib = ag.load_library()
    import ctypes

    dp = lambda tt: ctypes.cast(tt.data_ptr(), ctypes.POINTER(ctypes.c_double))
    rc = lib.axg_download(lat.handle, dp(h_phi), dp(h_phid), n * n, 0)
    assert rc == 0
    times = []
    for r in range(reps + 1):
        t_start = time.perf_counter()
        assert lib.axg_upload(lat.handle, dp(h_phi), dp(h_phid), n * n, 0) == 0
        assert lib.axg_leapfrog(lat.handle, t, dt, nsub, 1, 1) == 0
        assert lib.axg_download(lat.handle, dp(h_phi), dp(h_phid), n * n, 0) == 0
        times.append(time.perf_counter() - t_start)
        t += dt * nsub
    per = float(np.median(times[1:]))
    per_min = float(np.min(times[1:]))
    bytes_each = 2 * n ** 3 * 16
    # three more intervals split into their calls (each returns synchronised); medians
    parts = []
    for _ in range(3):
        t0 = time.perf_counter()
        assert lib.axg_upload(lat.handle, dp(h_phi), dp(h_phid), n * n, 0) == 0
        t1 = time.perf_counter()
        assert lib.axg_leapfrog(lat.handle, t, dt, nsub, 1, 1) == 0
        lat.synchronize()
        t2 = time.perf_counter()
        assert lib.axg_download(lat.handle, dp(h_phi), dp(h_phid), n * n, 0) == 0
        t3 = time.perf_counter()
        parts.append((t1 - t0, t2 - t1, t3 - t2))
        t += dt * nsub
    up, lf, dn = (float(np.median([q[i] for q in parts])) for i in range(3))
    split = {"upload_s": up, "leapfrog_s": lf, "download_s": dn, "upload_gbs": bytes_each / up / 1e9,
             "download_gbs": bytes_each / dn / 1e9}
    # the host link on its own: a plain pinned copy of phi's host buffer each
    # way (best of 3, CUDA events); upload + steps + download cannot beat
    # bytes / link rate + the device-side steps
    d_tmp = torch.empty(shape, dtype=torch.float64, device="cuda")
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    link = {}
    for name, dst, src in (("h2d_gbs", d_tmp, h_phi), ("d2h_gbs", h_phi, d_tmp)):
        best = 1e30
        for _ in range(3):
            ev[0].record()
            dst.copy_(src, non_blocking=True)
            ev[1].record()
            ev[1].synchronize()
            best = min(best, ev[0].elapsed_time(ev[1]) * 1e-3)
        link[name] = bytes_each / 2 / best / 1e9
    del d_tmp
    bound = bytes_each / (link["h2d_gbs"] * 1e9) + lf + bytes_each / (link["d2h_gbs"] * 1e9)
    split["link"] = link
    split["interval_bound_s"] = bound
    split["frac_of_link_bound"] = bound / per
    return {"value": nsub * n ** 3 / per, "unit": UNIT, "h2d_bytes_per_step": bytes_each / nsub,
            "d2h_bytes_per_step": bytes_each / nsub, "interval_steps": nsub, "s_per_interval": per,
            "s_per_interval_min": per_min, "split": split,
            "note": "public C-ABI, host-resident complex128 phi and phidot uploaded and downloaded "
                    "once per interval of %d leapfrog steps (pinned host memory); u_ij device-resident" % nsub}


ENSEMBLE_SIZES = [(64, 32), (128, 32), (160, 24), (192, 8)]  # (N, members): 96 realisations


def bench_ensemble(ag, steps, device, sizes=ENSEMBLE_SIZES):
    """Config 3: 96 seeded realisations of uneven sizes stepped together, one
    launch per step, intervals replayed from a CUDA graph."""
    ps = []
    for n, cnt in sizes:
        for r in range(cnt):
            ps.append(ag.default_params(ngrid=n, precision=ag.PREC_FP32_MIXED, gw_mode=ag.GW_UIJ,
                                        potential=ag.POT_REFERENCE, dspa=0.5, sigma_cr=1.0, kappa=0.1,
                                        seed=1 + len(ps), device=device))
    sites = sum(n ** 3 * c for n, c in sizes)
    t_setup = time.perf_counter()
    ens = ag.Ensemble(ps)
    try:
        for i, m in enumerate(ens.members):
            m.ic_gaussian_flat(2.0 * np.pi / (8 * 0.5), i)
        best, _ = ens.autotune(2)
        setup_s = time.perf_counter() - t_setup
        dt, interval = 0.05, max(1, steps // 4)
        t = 2.0
        # open the DKD sequence with its half drift, then time kick+drift steps
        # only (as the single-lattice line does); the interval graph is
        # captured on the first open-ended call and replayed after that
        ens.leapfrog(t, dt, 1, True, False)
        t += dt * 1.5
        ens.leapfrog(t, dt, interval, False, False)  # eager + capture
        t += dt * interval
        ens.leapfrog(t, dt, interval, False, False)  # replay (warm)
        t += dt * interval
        l0 = ens.launch_count()
        t_start = time.perf_counter()
        for _ in range(4):
            ens.leapfrog(t, dt, interval, False, False)
            t += dt * interval
        wall = time.perf_counter() - t_start
        launches = ens.launch_count() - l0
        nsteps = 4 * interval
        # the outputs of the 96-realisation workload: mean GW spectrum and mean
        # string / wall parameters over all members, each from the member's own call
        t_out = time.perf_counter()
        w, pm, pse, de = ens.grav_spec_mean(t)
        t_spec = time.perf_counter() - t_out
        t_out = time.perf_counter()
        xm, xse, am, ase = ens.defect_mean(1, t)
        t_def = time.perf_counter() - t_out
        outputs = {"tau": t, "gw_power_mean": [float(v) for v in pm], "gw_power_sem": [float(v) for v in pse],
                   "gw_bin_centres": [float(v) for v in w], "gw_modes": [float(v) for v in de],
                   "xi_mean": [float(v) for v in xm], "xi_sem": [float(v) for v in xse],
                   "wall_A_mean": [float(v) for v in am], "wall_A_sem": [float(v) for v in ase],
                   "gw_spectrum_s": t_spec, "id_defects_s": t_def,
                   "note": "means over all members of each member's own grav_spec_estimation and id_defects "
                           "(xi = (tau/dx)^2 sl / N^3 / 4, A = (tau/dx) wa / N^3 / 2, evolve.f90:191-192)"}
        return {"members": len(ps), "sizes": {f"{n}^3": c for n, c in sizes}, "sites": sites,
                "value": sites * nsteps / wall, "unit": UNIT, "ms_per_step": 1e3 * wall / nsteps,
                "steps": nsteps, "intervals": 4, "graph": True, "launches": launches,
                "batched_launches_per_step": 1, "tile": ens.members[0].tiles()[best],
                "launch_mode": "persistent CTAs" if ens.launch_mode() else "one CTA per work item",
                "setup_s": setup_s, "outputs": outputs,
                "timing": "host wall clock around graph replays of kick+drift steps (each call synchronises)"}
    finally:
        ens.close()


def bench_adjoint(ag, device, n=256, steps=2000, stride=64, fp64_steps=256):
    """The 256^3 gradient workload: J = GW energy of u_ij over k in
    [m_r/8, m_r/2] after `steps` leapfrog steps from tau = 1 (dt = 0.2), its
    gradient with respect to lambda and the initial fields by the
    hand-written adjoint (checkpoint every `stride` steps), and the cost of
    forward + reverse against a plain forward run of the same steps.  FP32-mixed
    (the workload's precision) at full length; FP64-plain on a shorter run."""
    out = {"n": n, "stride": stride, "timing": "CUDA events on the library stream"}
    for name, prec, st in (("fp32_mixed", ag.PREC_FP32_MIXED, steps), ("fp64_plain", ag.PREC_FP64_PLAIN, fp64_steps)):
        # sigma_cr = 0.005: dt = 0.2 stays inside the leapfrog's stability limit
        # (dt^2 (12/dx^2 + 6 tau^2 sigma_cr^2) < 4) over the 2000-step run to tau ~ 400
        p = ag.default_params(ngrid=n, precision=prec, gw_mode=ag.GW_UIJ, potential=ag.POT_QUARTIC,
                              dspa=1.0, sigma_cr=0.005, vev=1.0, seed=1, device=device, **{"lambda": 1.0})
        t1, dt = 1.0, 0.2
        with ag.Lattice(p) as lat:
            lat.ic_gaussian_flat(kcut=1.0, realisation=0)
            lat.leapfrog(t1, dt, 4, True, True)  # warm-up (plans, tensor maps, first launches)
            lat.ic_gaussian_flat(kcut=1.0, realisation=0)
            lat.synchronize()
            lat.event_record(0)
            lat.leapfrog(t1, dt, st, True, True)
            lat.event_record(1)
            plain = lat.event_elapsed(0, 1)
            lat.ic_gaussian_flat(kcut=1.0, realisation=0)
            J, dl, _, _, mf, mr = lat.adjoint_gw_band(t1, dt, st, stride, 0.125, 0.5, want_grads=False)
            # per-kernel breakdown on a shorter run (launch events add overhead)
            lat.ic_gaussian_flat(kcut=1.0, realisation=0)
            lat.set_kernel_timing(True)
            kst = min(st, 256)
            lat.adjoint_gw_band(t1, dt, kst, stride, 0.125, 0.5, want_grads=False)
            kt = lat.kernel_timings()
            lat.set_kernel_timing(False)
        out[name] = {"steps": st, "J": J, "dJ_dlambda": dl, "ms_forward_step": plain / st,
                     "ms_forward_with_checkpoints": mf, "ms_reverse": mr, "reverse_vs_forward": mr / plain,
                     "adjoint_total_vs_forward": (mf + mr) / plain,
                     "kernels_ms_per_step": {k: round(t / kst, 4) for k, l, t in kt if l > 0}}
    return out


def bench_output_calls(ag, n, device, steps=200, max_fit_cells=40_000_000):
    """Per-call cost of the output-time routines on the evolved FP32-mixed
    lattice (host wall clock around each call; every call synchronises):
    plaquette winding, cell classification, defect fits and sums, field
    spectrum with window deconvolution, u_ij GW spectra (linear and log
    bins).  Defect fits are skipped above max_fit_cells string+wall cells."""
    p = workload_params(ag, n, ag.PREC_FP32_MIXED, ag.GW_UIJ, device)
    out = {"n": n, "evolved_steps": steps, "timing": "host wall clock, each call synchronises"}
    with ag.Lattice(p) as lat:
        lat.ic_gaussian_flat(kcut=2.0 * np.pi / (8 * p.dspa))
        dt, _ = lat.get_dtau(2.0, 32.0, 0.25)
        lat.leapfrog(2.0, dt, steps, True, True)
        tau = 2.0 + dt * steps
        out["tau"] = tau

        def timed(name, fn, reps=3, warm=True):
            if warm:
                fn()  # first call allocates plans / tables
            lat.set_kernel_timing(True)
            t0 = time.perf_counter()
            for _ in range(reps):
                r = fn()
            out[name] = {"ms": 1e3 * (time.perf_counter() - t0) / reps}
            kt = lat.kernel_timings()
            lat.set_kernel_timing(False)
            out[name]["kernels_ms"] = {k: round(t / reps, 3) for k, l, t in kt if l > 0}
            return r

        wind = timed("string_winding", lat.string_winding)
        counts = timed("classify_cells", lambda: lat.classify_cells(7))
        out["string_winding"]["plaquettes"] = [int(c) for c in wind]
        out["classify_cells"]["counts"] = [int(c) for c in counts]
        cells = int(counts[0] + counts[1])
        if cells <= max_fit_cells:
            r = timed("id_defects", lambda: lat.id_defects(1, tau), reps=1, warm=False)
            out["id_defects"]["fitted_cells"] = cells
            out["id_defects"]["cells_per_s"] = cells / (out["id_defects"]["ms"] * 1e-3)
        else:
            out["id_defects"] = {"skipped": f"{cells} string+wall cells above the {max_fit_cells} cap"}
        timed("spectrum_estimation", lambda: lat.spectrum_estimation(tau))
        # fit throughput on a 128^3 lattice of the same physics and age
        p128 = workload_params(ag, 128, ag.PREC_FP32_MIXED, ag.GW_UIJ, device)
        with ag.Lattice(p128) as small:
            small.ic_gaussian_flat(kcut=2.0 * np.pi / (8 * p128.dspa))
            dt128, _ = small.get_dtau(2.0, 32.0, 0.25)
            nst = int(round((tau - 2.0) / dt128))
            small.leapfrog(2.0, dt128, nst, True, True)
            c128 = small.classify_cells(7)
            small.set_kernel_timing(True)
            t0 = time.perf_counter()
            small.id_defects(1, 2.0 + dt128 * nst)
            ms = 1e3 * (time.perf_counter() - t0)
            kt = small.kernel_timings()
            small.set_kernel_timing(False)
            out["id_defects_128"] = {"ms": ms, "string_cells": int(c128[0]), "wall_cells": int(c128[1]),
                                     "cells_per_s": float(c128[0] + c128[1]) / (ms * 1e-3),
                                     "kernels_ms": {k: round(t, 3) for k, l, t in kt if l > 0}}
        timed("grav_spec_estimation", lambda: lat.grav_spec_estimation(tau))
        timed("grav_spec_log", lambda: lat.grav_spec_log(tau))
    return out


def bench_config2(ag, device, n=1024, steps=200, every=10, gw_outputs=8):
    """The 1024^3 FP32-mixed workload: phi and six u_ij, quartic potential
    (lambda = v = 1, dx = 1, sigma_cr = 0.005), the axion term
    m_a^2 (tau / tau_on)^2 (1 - cos N_DW theta) / N_DW^2 switched on half-way
    through the run, N_DW = 1 and 2; string and wall classification and the
    plaquette winding every `every` steps, the GW spectrum (linear and log
    bins) at `gw_outputs` output times.  Steps are timed with CUDA events on
    the library's stream, output calls with the host clock (each ends with a
    synchronising download of its result)."""
    try:
        import torch

        free = torch.cuda.mem_get_info(device)[0]
    except Exception:
        free = None
    if free is not None and free < 200 * 2 ** 30:
        return {"skipped": f"needs ~200 GiB of free device memory, {free / 2 ** 30:.0f} GiB free"}
    t0, dt = 10.0, 0.2
    nout = steps // every
    gw_at = {int(round(nout * (k + 1) / gw_outputs)) for k in range(gw_outputs)}
    res = {"n": n, "steps": steps, "defects_every": every, "gw_outputs": sorted(gw_at), "tau_start": t0, "dt": dt}
    for ndw in (1, 2):
        tau_on = t0 + dt * steps / 2
        p = ag.default_params(ngrid=n, precision=ag.PREC_FP32_MIXED, gw_mode=ag.GW_UIJ, potential=ag.POT_QUARTIC,
                              dspa=1.0, sigma_cr=0.005, vev=1.0, n_dw=ndw, ma2_0=1e-3, tau_axion_on=tau_on,
                              ma2_power=2.0, seed=1, gw_log_bins=64, flags=7, device=device, **{"lambda": 1.0})
        w0 = time.perf_counter()
        with ag.Lattice(p) as lat:
            lat.ic_gaussian_flat(kcut=1.0)
            step_ms, cls_s, wind_s, gw_s, counts, winds = 0.0, [], [], [], [], []
            t = t0
            for k in range(1, nout + 1):
                lat.event_record(0)
                lat.leapfrog(t, dt, every, True, True)
                lat.event_record(1)
                step_ms += lat.event_elapsed(0, 1)
                t += dt * every
                c0 = time.perf_counter()
                c = lat.classify_cells(7)
                cls_s.append(time.perf_counter() - c0)
                c0 = time.perf_counter()
                wnd = lat.string_winding()
                wind_s.append(time.perf_counter() - c0)
                counts.append([int(x) for x in c])
                winds.append(int(wnd.sum()))
                if k in gw_at:
                    c0 = time.perf_counter()
                    lat.grav_spec_estimation(t)
                    lat.grav_spec_log(t)
                    gw_s.append(time.perf_counter() - c0)
        res[f"n_dw_{ndw}"] = {
            "tau_axion_on": tau_on, "tau_end": t, "wall_s": time.perf_counter() - w0,
            "step_ms": step_ms / steps, "classify_ms": 1e3 * float(np.median(cls_s)),
            "winding_ms": 1e3 * float(np.median(wind_s)), "gw_spectra_ms": 1e3 * float(np.median(gw_s)),
            "string_wall_mask_counts_first_last": [counts[0], counts[-1]],
            "pierced_plaquettes_first_last": [winds[0], winds[-1]],
            "site_updates_per_s": float(n) ** 3 / (step_ms / steps * 1e-3)}
    return res


def accuracy_fp32(ag, n, steps, device):
    """GW (u_ij TT) spectrum and field moments of the FP32-mixed path against
    the FP64-plain path (bit-identical to the FP64 CPU restatement) after the
    same evolution from the same initial state."""
    out = {}
    res = {}
    for name, prec in (("fp64", ag.PREC_FP64_PLAIN), ("fp32", ag.PREC_FP32_MIXED)):
        p = workload_params(ag, n, prec, ag.GW_UIJ, device)
        with ag.Lattice(p) as lat:
            lat.ic_gaussian_flat(kcut=2.0 * np.pi / (8 * p.dspa))
            dt, _ = lat.get_dtau(2.0, 32.0, 0.25)
            lat.leapfrog(2.0, dt, steps, True, True)
            tau = 2.0 + dt * steps
            w, pw, nu, de = lat.grav_spec_estimation(tau)
            e, lpw, lnu, lde = lat.grav_spec_log(tau)
            mom = lat.field_moments(tau)
            counts = lat.classify_cells(7)
            res[name] = (nu, lnu, mom, counts)
    nu64, lnu64, m64, c64 = res["fp64"]
    nu32, lnu32, m32, c32 = res["fp32"]
    ok = nu64 > 0
    okl = lnu64 > 0
    out["gw_linear_bins_max_rel_err"] = float(np.max(np.abs(nu32[ok] - nu64[ok]) / nu64[ok])) if ok.any() else None
    out["gw_log_bins_max_rel_err"] = float(np.max(np.abs(lnu32[okl] - lnu64[okl]) / lnu64[okl])) if okl.any() else None
    out["moments_rel_err"] = [float(abs(a - b) / abs(b)) if b != 0 else None for a, b in zip(m32, m64)]
    out["defect_counts_fp32"] = [int(x) for x in c32]
    out["defect_counts_fp64"] = [int(x) for x in c64]
    out["n"] = n
    out["steps"] = steps
    out["note"] = ("same seeded IC evolved by both paths; FP64-plain is bit-identical to the FP64 CPU restatement "
                   "(tests); errors are per bin of the shell-summed |W'_TT|^2 + k^2|W_TT|^2")
    return out


def cpu_oracle_rate(n, steps, threads=None, warmup=1):
    """FP64 CPU restatement of evolve.f90 (phi + six u_ij), all host threads."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import axo  # the oracle's own parameter defaults: no GPU library is loaded

    p = axo.default_params(ngrid=n, precision=0, gw_mode=2, dspa=32.0 / n, **WORKLOAD_KW)
    # the GPU arm's initial state: the same seeded Gaussian-flat field
    phi, phid = axo.ic_gaussian_flat(p, kcut=2.0 * np.pi / (8 * p.dspa))
    u = np.zeros((6, n, n, n))
    ud = np.zeros((6, n, n, n))
    dt, _ = axo.get_dtau(p, 2.0, 32.0, 0.25)
    axo.leapfrog(p, phi, phid, u, ud, None, 2.0, dt, 1, True, False)  # opens the DKD sequence (warm-up)
    t = 2.0 + 1.5 * dt
    for _ in range(max(0, warmup - 1)):
        axo.leapfrog(p, phi, phid, u, ud, None, t, dt, 1, False, False)
        t += dt
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        axo.leapfrog(p, phi, phid, u, ud, None, t, dt, 1, False, False)
        times.append(time.perf_counter() - t0)
        t += dt
    per = float(np.median(times))
    return n ** 3 / per, per, axo.lib().axo_num_threads()


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return
    n = args.n
    steps = max(1, args.steps)
    warm = max(1, args.warmup)
    rate, per, cores = cpu_oracle_rate(n, steps, warmup=warm)
    sample = f"{steps} leapfrog steps (phi + 6 u_ij, FP64) of the {n}^3 lattice after {warm} warm-up steps"
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": world,
        "steps": steps, "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(n), "n": n, "gw_mode": "uij", "precision": "fp64",
                   "parallelism": f"OpenMP x{cores} (rank 0 only)",
                   "implementation": "CPU restatement of evolve.f90 (oracle/, C + OpenMP, FP64); the Fortran "
                                     "reference needs ifort/MPI/MKL/FFTW, none present"},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64-plain comparison arm")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--e2e-interval", type=int, default=20)
    ap.add_argument("--e2e-reps", type=int, default=15,
                    help="timed upload + steps + download intervals (median; robust to a burst of host-link traffic)")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the batched-ensemble measurement")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP32-vs-FP64 accuracy block")
    ap.add_argument("--accuracy-steps", type=int, default=100)
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint-gradient cost block")
    ap.add_argument("--no-phi-only", action="store_true", help="skip the phi-only (no u_ij) figures")
    ap.add_argument("--no-green", action="store_true", help="skip the Green's-function GW mode step cost")
    ap.add_argument("--no-output-calls", action="store_true", help="skip the defect / spectrum call timings")
    ap.add_argument("--ensemble-sizes", default=None,
                    help="ensemble members as N:count,... (default 64:32,128:32,160:24,192:8, the 96 realisations)")
    ap.add_argument("--tile", type=int, default=None,
                    help="fused-kernel tile index (axg_tile_info) instead of autotuning the headline arm")
    ap.add_argument("--adjoint-steps", type=int, default=2000)
    ap.add_argument("--no-config2", action="store_true", help="skip the 1024^3 axion-term workload block")
    ap.add_argument("--config2-steps", type=int, default=200,
                    help="leapfrog steps of the 1024^3 workload (2560 reach tau ~ L / 2)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    if args.impl == "reference":
        run_reference(args)
        return

    rank, world, local = env_rank()
    dist = None
    if world > 1:
        import torch.distributed as tdist

        backend = "nccl" if os.environ.get("AXG_BENCH_GLOO") is None else "gloo"
        tdist.init_process_group(backend=backend)
        dist = tdist
    import torch

    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    import axion_grav_gb300 as ag

    n = args.n
    r32 = bench_ours(ag, n, ag.PREC_FP32_MIXED, ag.GW_UIJ, args.steps, args.warmup, dist, local, clocks=True,
                     tile=args.tile)
    lat = r32.pop("lat")
    e2e = bench_e2e(ag, lat, n, args.e2e_interval, args.e2e_reps, r32["t"], r32["dt"]) if rank == 0 else None
    lat.close()

    ms = replica_time_ms(r32["ms"], dist)
    sites = float(n) ** 3
    value = job_rate(world, sites, args.steps, ms)

    peak, peak_kind = measured_peaks()
    kern = {k: (l, t) for k, l, t in r32["kernels"]}
    dom = max(kern, key=lambda k: kern[k][1])
    l, tot = kern[dom]
    avg_ms = tot / max(l, 1)
    alg = BYTES_PER_SITE.get(dom, 0) * sites
    achieved = alg / (avg_ms * 1e-3) / 1e9
    tps = ncu_traffic_per_site(dom)
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": tps * sites if tps is not None else None, "kernel": dom,
            "algorithmic_bytes_per_launch": alg, "avg_launch_ms": avg_ms,
            "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)" if peak_kind == "measured" else "fallback 6.8 TB/s"}

    fp64 = None
    if not args.no_fp64:
        r64 = bench_ours(ag, n, ag.PREC_FP64_PLAIN, ag.GW_UIJ, max(3, args.steps // 8), args.warmup, dist, local)
        r64.pop("lat").close()
        k64 = {k: (l, t) for k, l, t in r64["kernels"]}
        st64 = max(3, args.steps // 8)
        v64 = job_rate(world, sites, st64, replica_time_ms(r64["ms"], dist))
        byts = sum(BYTES_PER_SITE.get(k, 0) * sites * l for k, (l, t) in k64.items())
        tms = sum(t for k, (l, t) in k64.items())
        fp64 = {"value": v64, "ms_per_step": r64["ms"] / st64, "steps": st64,
                "kernels": {k: {"launches": l, "avg_ms": t / max(l, 1)} for k, (l, t) in k64.items()},
                "hbm_frac": (byts / (tms * 1e-3) / 1e9) / peak if tms > 0 else None,
                "fp32_mixed_speedup": value / v64 / world * world}

    # FP64-fused: the TMA kernel doing the plain path's FP64 operations in the
    # same order (bit-identical results), one pass per step
    if fp64 is not None:
        st64f = max(3, args.steps // 8)
        rf = bench_ours(ag, n, ag.PREC_FP64_FUSED, ag.GW_UIJ, st64f, args.warmup, dist, local)
        rf.pop("lat").close()
        kf = {k: (l, t) for k, l, t in rf["kernels"]}
        fp64["fused"] = {"value": job_rate(world, sites, st64f, replica_time_ms(rf["ms"], dist)),
                         "ms_per_step": rf["ms"] / st64f, "steps": st64f, "tile": rf["tile_shape"],
                         "kernels": {k: {"launches": l, "avg_ms": t / max(l, 1)} for k, (l, t) in kf.items()}}

    green = None
    if not args.no_green:
        green = {}
        for name, prec in (("fp32_mixed", ag.PREC_FP32_MIXED), ("fp64_plain", ag.PREC_FP64_PLAIN)):
            st = max(3, args.steps // 20)
            r = bench_ours(ag, n, prec, ag.GW_GREEN, st, args.warmup, dist, local)
            r.pop("lat").close()
            kk = {k: (l, t) for k, l, t in r["kernels"]}
            green[name] = {"ms_per_step": r["ms"] / st, "steps": st,
                           "value": job_rate(world, sites, st, replica_time_ms(r["ms"], dist)),
                           "kernels": {k: {"launches": l, "avg_ms": t / max(l, 1)} for k, (l, t) in kk.items()}}

    phi_only = None
    if not args.no_phi_only:
        phi_only = {}
        for name, prec, st in (("fp32_mixed", ag.PREC_FP32_MIXED, args.steps),
                               ("fp64_plain", ag.PREC_FP64_PLAIN, max(3, args.steps // 4))):
            r = bench_ours(ag, n, prec, ag.GW_NONE, st, args.warmup, dist, local)
            r.pop("lat").close()
            kk = {k: (l, t) for k, l, t in r["kernels"]}
            byts = sum(BYTES_PER_SITE_PHI_ONLY.get(k, BYTES_PER_SITE.get(k, 0)) * sites * l for k, (l, t) in kk.items())
            tms = sum(t for k, (l, t) in kk.items())
            phi_only[name] = {"value": job_rate(world, sites, st, replica_time_ms(r["ms"], dist)),
                              "ms_per_step": r["ms"] / st, "steps": st,
                              "hbm_frac": (byts / (tms * 1e-3) / 1e9) / peak if tms > 0 else None,
                              "tile": r["tile_shape"]}

    ensemble = None
    if not args.no_ensemble:
        try:
            sizes = ENSEMBLE_SIZES
            if args.ensemble_sizes:
                sizes = [tuple(int(v) for v in part.split(":")) for part in args.ensemble_sizes.split(",")]
            ensemble = bench_ensemble(ag, max(8, args.steps // 2), local, sizes)
        except Exception as exc:
            ensemble = {"error": str(exc)}
    accuracy = None
    if rank == 0 and not args.no_accuracy:
        try:
            accuracy = accuracy_fp32(ag, n, args.accuracy_steps, local)
        except Exception as exc:
            accuracy = {"error": str(exc)}

    output_calls = None
    if rank == 0 and not args.no_output_calls:
        try:
            output_calls = bench_output_calls(ag, n, local)
        except Exception as exc:
            output_calls = {"error": str(exc)}

    adjoint = None
    if rank == 0 and not args.no_adjoint:
        try:
            adjoint = bench_adjoint(ag, local, steps=args.adjoint_steps)
        except Exception as exc:
            adjoint = {"error": str(exc)}

    config2 = None
    if rank == 0 and not args.no_config2:
        try:
            config2 = bench_config2(ag, local, steps=args.config2_steps)
        except Exception as exc:
            config2 = {"error": str(exc)}

    cpu = None
    if rank == 0 and not args.no_cpu:
        try:
            rate, per, cores = cpu_oracle_rate(n, args.cpu_steps)
            cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                   "sample": f"{args.cpu_steps} leapfrog steps (phi + 6 u_ij, FP64) of the {n}^3 lattice, "
                             f"CPU restatement of evolve.f90 (oracle/), OpenMP"}
        except Exception as exc:  # the baseline is reported, never required
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                   "sample": f"failed: {exc}"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload_name(n),
                       "n": n, "gw_mode": "uij", "precision": "fp32_mixed", "parallelism": f"replicas x{world}",
                       "implementation": "FP32-mixed fused TMA kernel with Kahan-compensated drifts (libaxgpu.so)",
                       "l2": "no flush: state %.1f GiB >> 126 MB L2" % (sites * 96 / 2 ** 30),
                       "tile": r32["tile_shape"]},
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": r32["launches"],
            "clocks": r32["clocks"], "adjoint": adjoint, "phi_only": phi_only, "green": green,
            "output_calls": output_calls, "axion_1024": config2,
            # last, so that a reader keeping only the tail of the line sees them
            "ensemble": ensemble, "accuracy": accuracy, "fp64_plain": fp64,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
