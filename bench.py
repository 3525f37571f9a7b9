#!/usr/bin/env python
"""Benchmark: 3-D vortex Navier-Stokes steps/s at NR x NP x NZ = 192 x 128 x 128 on one GB300.

Workload (the metric's configuration): Batchelor q-vortex (q = 4) at the origin built by the
reference's qvort_dist_tp recipe, Re = 1e4 (visc = 1e-4), ELL = 4, full chops (NRCHOP=192,
NPCHOP=65, NZCHOP=65), dt = 1e-3, SVV filter on with the reference defaults, background u_z = 0,
plus a seeded perturbation of amplitude 1e-4 on the (psi, chi) coefficients with |m| <= 4, |k| <= 8.
A step is one main-loop iteration of src/apps/vortical_flow_3d.f90 (abcn x2, dealias, svv_filter,
zeroat1, advection_rhs, check_stability).  Data: synthetic (seeded); every field is 26 MB and the
step touches ~20 of them, so the working set exceeds the 129 MB L2 and no flush is needed.

Arms:
  default          the GPU library (mixed form timed as `value`; the plain FP64 form timed beside it,
                   with the relative error of mixed against FP64 per field)
  --impl reference the reference's CPU path for this workload: the oracle port (C++ restatement of
                   the Fortran, OpenMP over the host cores), since the Fortran reference cannot be
                   built here (no Fortran compiler / MPI / LAPACK)
Under torchrun (N > 1) every rank runs an independent replica on its own GPU (the path does not
shard on one GPU per box: replicas only); value = total steps/s over ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(nr=192, np=128, nz=128, nrchop=192, npchop=65, nzchop=65, ell=4.0, visc=1.0e-4)
DT = 1.0e-3
Q = 4.0
PERT = 1.0e-4
METRIC = "steps/s @192x128x128 (3-D vortex NS step, mixed precision on GPU)"
# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the step's largest kernels, from
# one ncu capture of `bench.py --profile-run` at this workload (profiles/)
NCU_TRAFFIC = {"k_band_subst<2>": 104.9e6, "k_band_subst<1>": 93.5e6, "k_xs_rtrans<1, 6, 16>": 85.8e6}


def workload_params():
    from mlegs_gb300.params import make_params
    return make_params(**WORKLOAD)


def perturbation(p, dims):
    from mlegs_gb300 import fields
    return (fields.spectral_noise(p, dims, 1001, amp=PERT, decay=0.3, m_max=4, k_max=8),
            fields.spectral_noise(p, dims, 1002, amp=PERT, decay=0.3, m_max=4, k_max=8))


def config_dict():
    return {"workload": "vortex3d NR=192 NP=128 NZ=128 ELL=4 NRCHOP=192 NPCHOP=65 NZCHOP=65 q=4 Re=1e4 dt=1e-3 "
                        "SVV on, perturbation 1e-4 |m|<=4 |k|<=8",
            "field_MB": 195 * 65 * 128 * 16 / 1e6,
            "l2_policy": "inputs larger than L2 (working set ~20 fields x 26 MB), no flush"}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader",
                                          "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1].split()[0]))
                smax.append(float(f[2].split()[0]))
            except ValueError:
                continue
            for name, v in zip(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"], f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if os.environ.get("MLG_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return rank, world, local, pg


def max_over_ranks(pg, ms):
    """The slowest rank's time: replicas run concurrently, the job ends with the last one."""
    if pg is None:
        return ms
    import torch
    dev = "cuda" if pg.get_backend() == "nccl" else "cpu"
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def job_steps_per_s(world, steps, ms):
    """Whole-job throughput: every rank advanced its own replica by `steps` in `ms` (max over ranks)."""
    return world * steps / (ms / 1e3)


def run_reference(args, rank, world, pg):
    """The reference arm: the CPU path (oracle port) on this host's cores, rank 0 only."""
    if rank != 0:
        return
    from oracle.oracle import Oracle
    from mlegs_gb300 import vortex
    threads = os.cpu_count() or 1
    p = workload_params()
    o = Oracle(p, threads=threads)
    st = vortex.VortexState(o)
    vortex.qvort_init(o, st, q=Q, uz_b=0.0, pert=perturbation(p, o.dims))
    # untimed start-up: one advection_rhs and the history copies (the cost of a step does not depend
    # on whether the Richardson start-up ran)
    o.advection_rhs(st.psi, st.chi, st.nlpsi, st.nlchi, st.uz)
    for a, b in (("psi_p", "psi"), ("chi_p", "chi"), ("nlpsi_p", "nlpsi"), ("nlchi_p", "nlchi")):
        getattr(st, a).copy_from(getattr(st, b))
    t0 = time.perf_counter()
    for _ in range(max(args.warmup, 1) if args.warmup else 1):
        vortex.step(o, st, DT)
        if time.perf_counter() - t0 > 60:
            break
    per = (time.perf_counter() - t0) / max(args.warmup, 1)
    # a bounded sample: at most ~90 s of CPU work, at least one step
    k = max(1, min(args.steps, int(90.0 / max(per, 1e-3))))
    t0 = time.perf_counter()
    for _ in range(k):
        vortex.step(o, st, DT)
    dt_s = time.perf_counter() - t0
    value = k / dt_s
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world,
            "steps": k, "warmup": args.warmup, "ms_per_step": 1e3 * dt_s / k, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": config_dict(),
            "cpu_baseline": {"value": value, "unit": "steps/s", "cores": threads, "kind": "port",
                             "sample": f"{k} timed steps (of {args.steps} requested) after {args.warmup} warm-up, "
                                       "oracle C++ restatement with OpenMP"},
            "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def ke_spectrum(kit, st_fields, dims, xw):
    """Kinetic-energy spectrum E(m, k) of the velocity of (psi, chi) from the library's FP64 diagnostic
    (mlg_ke_spectrum): E(m, k) = 1/2 sum_i w_i r_i^2/(1 - x_i^2) 2 pi zlen c_m |u_hat(i, m, k)|^2 over
    the three components, u_hat the phi and z Fourier coefficients of the physical velocity, c_m = 2 for
    0 < m < np/2.  Sum over (m, k) = the kinetic energy."""
    psi = kit.scalar(*st_fields["psi"][:3])
    chi = kit.scalar(*st_fields["chi"][:3])
    E = kit.ke_spectrum(psi, chi)
    for s in (psi, chi):
        s.free()
    return E


def snapshot(st):
    return {n: getattr(st, n).get() for n in st.names}


def restore(st, snap):
    for n, (e, ln, sp, _) in snap.items():
        getattr(st, n).set(e, ln, sp)


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb else float(np.linalg.norm(a))


def run_ours(args, rank, world, local, pg):
    import torch
    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    from mlegs_gb300 import vortex
    from mlegs_gb300.kit import Kit, MIXED, PLAIN_FP64
    p = workload_params()
    with torch.cuda.stream(stream):
        t_init0 = time.perf_counter()
        kit = Kit(p, stream=stream.cuda_stream)
        kit.sync()
        t_init = time.perf_counter() - t_init0
        st = vortex.VortexState(kit)
        vortex.qvort_init(kit, st, q=Q, uz_b=0.0, pert=perturbation(p, kit.dims))
        vortex.bootstrap(kit, st, DT)
        kit.sync()
        snap0 = snapshot(st)

        def timed(mode, steps, warmup, clocks=None):
            kit.set_precision(mode)
            restore(st, snap0)
            st.gains = [0.0, 0.0]
            if warmup:
                kit.vortex_run(*st.args(), DT, warmup, st.gains)
            kit.sync()
            if pg:
                pg.barrier()
            torch.cuda.synchronize()
            if clocks:
                clocks.start()
            l0 = kit.launch_count()
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            kit.vortex_run(*st.args(), DT, steps, st.gains)
            ev1.record(stream)
            torch.cuda.synchronize()
            if pg:
                pg.barrier()
            ck = clocks.stop() if clocks else None
            ms = ev0.elapsed_time(ev1)
            return ms, kit.launch_count() - l0, ck

        clocks = Clocks(local)
        ms_mixed, launches, ck = timed(MIXED, args.steps, args.warmup, clocks)
        ms_mixed = max_over_ranks(pg, ms_mixed)
        value = job_steps_per_s(world, args.steps, ms_mixed)

        # plain FP64 over the same steps
        k_cmp = min(args.steps, 20)
        ms_plain, _, _ = timed(PLAIN_FP64, k_cmp, 2)
        plain_sps = k_cmp / (ms_plain / 1e3)
        # accuracy: both forms over the same accuracy_steps from the same state; per-field relative L2
        # of mixed against FP64 at the end, and the kinetic-energy spectrum error
        finals = {}
        for mode in (PLAIN_FP64, MIXED):
            kit.set_precision(mode)
            restore(st, snap0)
            st.gains = [0.0, 0.0]
            kit.vortex_run(*st.args(), DT, args.accuracy_steps, st.gains)
            kit.sync()
            finals[mode] = {n: getattr(st, n).get() for n in ("psi", "chi", "nlpsi", "nlchi")}
        err = {n: rel_l2(finals[MIXED][n][0], finals[PLAIN_FP64][n][0]) for n in finals[MIXED]}
        xw = (kit.kit_get("x"), kit.kit_get("w"), kit.kit_get("r"))
        E64 = ke_spectrum(kit, finals[PLAIN_FP64], kit.dims, xw)
        E32 = ke_spectrum(kit, finals[MIXED], kit.dims, xw)
        big = E64 > 1e-12 * E64.max()
        pert = np.ones_like(E64, dtype=bool)
        pert[0, 0] = False
        spec = {"max_rel_err": float(np.max(np.abs(E32 - E64)[big] / E64[big])),
                "rel_l2": rel_l2(E32, E64),
                "perturbation_max_rel_err": float(np.max(np.abs(E32 - E64)[big & pert] / E64[big & pert])),
                "modes_compared": int(big.sum()), "floor": "E > 1e-12 max E",
                "ke_total": float(E64.sum()), "ke_perturbation": float(E64[pert].sum())}

        # kernel classes timed launch by launch (CUDA events on the library's stream)
        kit.set_precision(MIXED)
        restore(st, snap0)
        kit.kernel_timing(True)
        kit.vortex_run(*st.args(), DT, 2, st.gains)
        kt = {name: kit.kernel_timing_read(i) for i, name in
              enumerate(["radial_fwd", "fft", "banded", "radial_bwd", "vec2tp", "solve"])}
        kit.kernel_timing(False)
        kit.sync()

        # end to end through the C ABI with host buffers: every step uploads psi and chi (e and ln)
        # from pinned host memory, steps, and downloads psi and chi into pinned host memory
        import ctypes
        from mlegs_gb300.kit import load
        L = load()
        kit.set_precision(MIXED)
        restore(st, snap0)
        dims = kit.dims
        host = [torch.empty(dims[::-1], dtype=torch.complex128, pin_memory=True).numpy().T for _ in range(2)]
        lns = [ctypes.c_double(0.0), ctypes.c_double(0.0)]
        sp = ctypes.create_string_buffer(4)
        for h, n, l in zip(host, ("psi", "chi"), lns):
            L.mlg_scalar_download(getattr(st, n).h, h.ctypes.data, ctypes.byref(l), sp)
        k_e2e = min(args.steps, 20)
        kit.sync()
        t0 = time.perf_counter()
        for _ in range(k_e2e):
            for h, n, l in zip(host, ("psi", "chi"), lns):
                L.mlg_scalar_upload(getattr(st, n).h, h.ctypes.data, l.value, b"FFF")
            kit.vortex_step(*st.args(), DT, st.gains)
            for h, n, l in zip(host, ("psi", "chi"), lns):
                L.mlg_scalar_download(getattr(st, n).h, h.ctypes.data, ctypes.byref(l), sp)
        e2e_s = time.perf_counter() - t0
        fbytes = int(np.prod(dims) * 16)

    if rank != 0:
        return
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    bf16 = peaks.get("bf16_tflops", 1900.0)
    # the dominant kernel class by time per step; its algorithmic work per launch is what the library
    # counts for it (bytes: each field read and written once, tables / factors read once)
    dom = max(kt, key=lambda n: kt[n][0])
    d_ms, d_n, d_work = kt[dom]
    avg_ms = d_ms / max(d_n, 1)
    nrc, npc, nz, nrh, nr = 192, 65, 128, 96, 192
    sum_nn = sum(max(nrc - m, 0) for m in range(npc))
    field_full = nr * npc * nz * 16          # rows < nr of every column m < npc (the physical side)
    field_spec = sum_nn * nz * 16            # rows < nn(m) (the spectral side)
    flops_field = 4.0 * sum_nn * nrh * nz    # one field's radial transform (complex x real MACs)
    # the exact-slice table images (mixed form, 42-bit: six BF16 digits per entry and parity, one
    # 128-row tile, K chunks of 16): read once per launch, from L2 after the first
    xs_table = npc * 1 * ((nrh + 15) // 16) * 2 * 6 * 128 * 16 * 2
    xv_table = (npc - 1) * 2 * ((nrh + 15) // 16) * (5 + 5 + 7) * 128 * 16 * 2

    def flop_class_bytes(name, flops, launches):
        """Algorithmic bytes per launch of a contraction class: the fields its launches transform (counted
        from its algorithmic flops, one field = flops_field), each read and written once, plus the table
        images once per launch."""
        if name in ("radial_fwd", "radial_bwd"):
            nf = flops / flops_field
            return (nf * (field_full + field_spec) + launches * xs_table) / max(launches, 1)
        if name == "vec2tp":
            nf = flops / (5 * flops_field)
            return (nf * (3 * field_full + 2 * field_spec) + launches * xv_table) / max(launches, 1)
        return None

    bytes_launch = flop_class_bytes(dom, d_work, d_n)
    if bytes_launch is None:
        bytes_launch = d_work / max(d_n, 1)
    achieved_gbs = bytes_launch / (avg_ms * 1e-3) / 1e9
    # DRAM traffic per launch of the class's kernels from one ncu capture at this workload
    # (dram__bytes_read.sum + dram__bytes_write.sum), and what limits them
    r_fields = kt["radial_bwd"][2] / flops_field / max(kt["radial_bwd"][1], 1)   # fields per backward launch
    ncu = {"solve": {"kernel": "k_band_subst<2> (psi and chi Helmholtz) + k_band_subst<1> (idel2)",
                     "traffic": (NCU_TRAFFIC["k_band_subst<2>"] + NCU_TRAFFIC["k_band_subst<1>"]) / 2,
                     "traffic_per_kernel": {k: NCU_TRAFFIC[k] for k in ("k_band_subst<2>", "k_band_subst<1>")},
                     "limit": "latency of each system's serial FP64 recurrence: 8320 systems x 2 parts x NR fields "
                              "are about one or two warps per SM sub-partition; the FP64 pipe at 48% (ncu); the "
                              "solves stay FP64 in both forms"},
           "radial_bwd": {"kernel": "k_xs_rtrans<1, 6, 16> (three fields per launch) + the m = 0 planes beside it",
                          "traffic": NCU_TRAFFIC["k_xs_rtrans<1, 6, 16>"] * r_fields / 3.0,
                          "traffic_per_kernel": {"k_xs_rtrans<1, 6, 16> (3 fields)": NCU_TRAFFIC["k_xs_rtrans<1, 6, 16>"]},
                          "limit": "integer work of the digit cuts and the order sums between mbarrier hand-offs "
                                   "(ALU pipe 39%, tensor pipe 15%, issue 39% active; ncu)"}}
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved_gbs, "peak": hbm, "unit": "GB/s",
            "frac": achieved_gbs / hbm, "traffic": ncu.get(dom, {}).get("traffic"),
            "avg_launch_us": 1e3 * avg_ms, "launches_per_step": d_n / 2,
            "algorithmic_bytes_per_launch": bytes_launch,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}
    if dom in ncu:
        roof["ncu_kernel"] = ncu[dom]["kernel"]
        roof["limit"] = ncu[dom]["limit"]
        if "traffic_per_kernel" in ncu[dom]:
            roof["traffic_per_kernel"] = ncu[dom]["traffic_per_kernel"]
    # the tensor-core Legendre transforms (backward: m >= 1 on tcgen05, the m = 0 planes beside it):
    # algorithmic flops 4 sum_m nn(m) nrh nz per field against the bf16 peak; the exact-slice scheme
    # issues 21 BF16 digit products per algorithmic MAC (six digits a side, orders below six)
    r_ms, r_n, r_flops = kt["radial_bwd"]
    r_avg = r_ms / max(r_n, 1)
    r_tf = (r_flops / max(r_n, 1)) / (r_avg * 1e-3) / 1e12
    r_bytes = flop_class_bytes("radial_bwd", r_flops, r_n)
    roof_tc = {"bound": "tensor", "kernel": "radial_bwd (k_xs_rtrans<1, 6, 16>: exact BF16 digit slices on tcgen05)",
               "achieved": r_tf, "peak": bf16, "unit": "TFLOP/s", "frac": r_tf / bf16, "avg_launch_us": 1e3 * r_avg,
               "bf16_digit_products_per_mac": 21, "fields_per_launch": r_fields,
               "algorithmic_flops_per_launch": r_flops / max(r_n, 1),
               "hbm_view": {"algorithmic_bytes_per_launch": r_bytes,
                            "achieved_gbs": r_bytes / (r_avg * 1e-3) / 1e9,
                            "frac": r_bytes / (r_avg * 1e-3) / 1e9 / hbm},
               "peak_source": "MEASURED_PEAKS.json bf16_tflops (of measured)"}
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_mixed / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "bf16 exact digit slices (42-bit radial, 35/49-bit projection) + f32 FFTs, f64 solves and state",
        "data": "synthetic (seeded)",
        "config": config_dict(),
        "fp64_plain": {"value": plain_sps, "unit": "steps/s", "steps": k_cmp,
                       "mixed_speedup": value / world / plain_sps},
        "mixed_vs_fp64": {"steps": args.accuracy_steps, "rel_l2": err, "ke_spectrum": spec,
                          "note": "FP64 form = the oracle to 1e-11 (nlchi 5e-11; GPU parity tests)"},
        "kit_init_s": t_init,
        "gpu_launches": int(launches),
        "gpu_launches_per_step": launches / args.steps,
        "roofline": roof,
        "roofline_tensor": roof_tc,
        "kernel_classes_ms_per_step": {n: v[0] / 2 for n, v in kt.items()},
        "kernel_classes_launches_per_step": {n: v[1] / 2 for n, v in kt.items()},
        "clocks": ck,
        "e2e": {"value": k_e2e / e2e_s, "unit": "steps/s", "h2d_bytes_per_step": 2 * fbytes,
                "d2h_bytes_per_step": 2 * fbytes, "steps": k_e2e},
        "mem_high_water_MB": kit.mem_high_water() / 1e6,
    }
    if not args.no_cpu_baseline and world == 1:
        from oracle.oracle import Oracle
        from mlegs_gb300 import vortex as vx
        threads = os.cpu_count() or 1
        o = Oracle(p, threads=threads)
        so = vx.VortexState(o)
        restore(so, snap0)
        t0 = time.perf_counter()
        nstep = 0
        while nstep < 1 or (time.perf_counter() - t0 < 15.0 and nstep < 5):
            vx.step(o, so, DT)
            nstep += 1
        cpu_s = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": nstep / cpu_s, "unit": "steps/s", "cores": threads, "kind": "port",
                                "sample": f"{nstep} steps of the same workload from the same state"}
        # the GPU's plain form over the same steps from the same state, against the oracle
        kit.set_precision(PLAIN_FP64)
        restore(st, snap0)
        st.gains = [0.0, 0.0]
        so_gains = list(so.gains)
        kit.vortex_run(*st.args(), DT, nstep, st.gains)
        kit.sync()
        line["plain_vs_oracle"] = {
            "steps": nstep,
            "rel_l2": {n: rel_l2(getattr(st, n).get()[0], getattr(so, n).get()[0]) for n in ("psi", "chi", "nlpsi", "nlchi")},
            "svv_gains_abs_diff": [abs(a - b) for a, b in zip(st.gains, so_gains)],
            "note": "GPU plain form vs the CPU oracle after the same steps from the same state (192x128x128)"}
        o.close()
    if not args.no_adjoint and world == 1:
        line["adjoint"] = adjoint_case(args)
    if not args.no_sweep and world == 1:
        line["transform_sweep"] = transform_sweep(args)
    if args.large and world == 1:
        line["large"] = large_case(args)
    print(json.dumps(line), flush=True)


SWEEP_WORKLOAD = dict(nr=256, np=256, nz=256, nrchop=256, npchop=129, nzchop=129, ell=4.0)
SWEEP_TRIPS, SWEEP_ORACLE_TRIPS = 50, 1


def transform_sweep(args):
    """Transform-only sweep, 256 x 256 x 256, ELL = 4, full chops: spectral coefficients with uniform
    phase and magnitude exp(-0.05(n+|m|+|k|)) (seeded, Hermitian at m = 0), 50 forward+backward round
    trips FFF -> PPP -> FFF in each form, timed with CUDA events.  Errors: each form against the FP64
    oracle after one round trip (coefficients and the physical field), and mixed against FP64 after
    50 round trips."""
    from mlegs_gb300 import fields
    from mlegs_gb300.kit import Kit, MIXED, PLAIN_FP64
    from mlegs_gb300.params import make_params
    import torch
    p = make_params(**SWEEP_WORKLOAD)
    kit = Kit(p, stream=torch.cuda.current_stream().cuda_stream)
    c0 = fields.spectral_noise(p, kit.dims, 7, amp=1.0, decay=0.05)
    out = {"workload": "256^3 ELL=4 full chops, |c| = exp(-0.05(n+|m|+|k|)), FFF->PPP->FFF round trips",
           "field_MB": float(np.prod(kit.dims) * 16 / 1e6)}
    res = {}
    for mode, tag in ((PLAIN_FP64, "fp64"), (MIXED, "mixed")):
        kit.set_precision(mode)
        s = kit.scalar(c0, 0.0, "FFF")
        kit.trans(s, "PPP")
        phys1 = s.e
        kit.trans(s, "FFF")
        one = s.e
        for _ in range(2):
            kit.trans(s, "PPP"); kit.trans(s, "FFF")
        s.set(c0, 0.0, "FFF")
        kit.sync()
        stream = torch.cuda.current_stream()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(SWEEP_TRIPS):
            kit.trans(s, "PPP"); kit.trans(s, "FFF")
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
        res[tag] = (phys1, one, s.e)
        out[tag] = {"round_trips_per_s": SWEEP_TRIPS / (ms / 1e3), "ms_per_round_trip": ms / SWEEP_TRIPS}
        s.free()
    kit.close()
    mixed50, fp6450 = res["mixed"][2], res["fp64"][2]
    out["mixed"]["vs_fp64_after_50"] = {"rel_l2": rel_l2(mixed50, fp6450),
                                        "max_rel": float(np.max(np.abs(mixed50 - fp6450)) / np.max(np.abs(fp6450)))}
    out["mixed"]["speedup_vs_fp64"] = out["mixed"]["round_trips_per_s"] / out["fp64"]["round_trips_per_s"]
    if not args.no_cpu_baseline:
        from oracle.oracle import Oracle
        o = Oracle(p, threads=os.cpu_count() or 1)
        so = o.scalar(c0, 0.0, "FFF")
        o.trans(so, "PPP")
        ophys = so.get()[0]
        o.trans(so, "FFF")
        oone = so.get()[0]
        o.close()
        for tag in ("fp64", "mixed"):
            ph, one, _ = res[tag]
            out[tag]["vs_oracle_one_trip"] = {
                "physical_rel_l2": rel_l2(ph, ophys), "physical_max_rel": float(np.max(np.abs(ph - ophys)) / np.max(np.abs(ophys))),
                "coeff_rel_l2": rel_l2(one, oone), "coeff_max_rel": float(np.max(np.abs(one - oone)) / np.max(np.abs(oone)))}
    return out


LARGE_WORKLOAD = dict(nr=512, np=512, nz=256, nrchop=512, npchop=257, nzchop=129, ell=6.0, visc=5.0e-5)
LARGE_DT, LARGE_Q, LARGE_STEPS, LARGE_ADJ_STEPS, LARGE_CKPT = 5.0e-4, 2.0, 200, 100, 20


def large_case(args):
    """512 x 512 x 256, ELL = 6, Batchelor q = 2 vortex, Re = 2e4, dt = 5e-4: 200 mixed steps (SVV on,
    the reference default) timed and compared with the FP64 form over the same steps; then the adjoint
    (SVV off, which it requires) over 100 steps with checkpoints every 20.  Reports steps/s, the error
    against FP64 and the memory high-water mark."""
    from mlegs_gb300 import fields, vortex
    from mlegs_gb300.kit import Kit, MIXED, PLAIN_FP64
    from mlegs_gb300.params import make_params
    import torch
    out = {"workload": "NR=512 NP=512 NZ=256 ELL=6 q=2 Re=2e4 dt=5e-4, perturbation 1e-4 |m|<=4 |k|<=8"}
    p = make_params(**LARGE_WORKLOAD)
    kit = Kit(p, stream=torch.cuda.current_stream().cuda_stream)
    st = vortex.VortexState(kit)
    pert = (fields.spectral_noise(p, kit.dims, 5001, amp=PERT, decay=0.3, m_max=4, k_max=8),
            fields.spectral_noise(p, kit.dims, 5002, amp=PERT, decay=0.3, m_max=4, k_max=8))
    vortex.qvort_init(kit, st, q=LARGE_Q, uz_b=0.0, pert=pert)
    kit.set_precision(MIXED)
    vortex.bootstrap(kit, st, LARGE_DT)
    kit.sync()
    snap = snapshot(st)
    fin = {}
    for mode, tag in ((MIXED, "mixed"), (PLAIN_FP64, "fp64")):
        kit.set_precision(mode)
        restore(st, snap)
        st.gains = [0.0, 0.0]
        kit.vortex_run(*st.args(), LARGE_DT, 3, st.gains)
        restore(st, snap)
        st.gains = [0.0, 0.0]
        kit.sync()
        stream = torch.cuda.current_stream()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        kit.vortex_run(*st.args(), LARGE_DT, LARGE_STEPS, st.gains)
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
        fin[tag] = {n: getattr(st, n).e for n in ("psi", "chi", "nlpsi", "nlchi")}
        out[tag] = {"steps": LARGE_STEPS, "steps_per_s": LARGE_STEPS / (ms / 1e3), "ms_per_step": ms / LARGE_STEPS}
    out["mixed"]["rel_l2_vs_fp64"] = {n: rel_l2(fin["mixed"][n], fin["fp64"][n]) for n in fin["mixed"]}
    out["mixed"]["speedup_vs_fp64"] = out["mixed"]["steps_per_s"] / out["fp64"]["steps_per_s"]
    out["mem_high_water_MB_forward"] = kit.mem_high_water() / 1e6
    kit.close()
    # the adjoint, SVV off
    p2 = make_params(**dict(LARGE_WORKLOAD, is_svv=0))
    kit = Kit(p2, precision=MIXED, stream=torch.cuda.current_stream().cuda_stream)
    st = vortex.VortexState(kit)
    vortex.qvort_init(kit, st, q=LARGE_Q, uz_b=0.0, pert=pert)
    t0 = time.perf_counter()
    J = kit.adjoint_run(st.psi, st.chi, st.uz, LARGE_DT, LARGE_ADJ_STEPS, LARGE_CKPT)
    t_fwd = time.perf_counter() - t0
    gp, gc = kit.scalar(), kit.scalar()
    t0 = time.perf_counter()
    kit.adjoint_run(st.psi, st.chi, st.uz, LARGE_DT, LARGE_ADJ_STEPS, LARGE_CKPT, gp, gc)
    t_adj = time.perf_counter() - t0
    g = gp.e
    out["adjoint_mixed"] = {"steps": LARGE_ADJ_STEPS, "checkpoint": LARGE_CKPT, "J": J, "forward_s": t_fwd,
                            "adjoint_run_s": t_adj, "sweep_over_forward": (t_adj - t_fwd) / t_fwd,
                            "gradient_finite": bool(np.all(np.isfinite(g))), "svv": "off"}
    out["mem_high_water_MB"] = kit.mem_high_water() / 1e6
    kit.close()
    return out


ADJ_WORKLOAD = dict(nr=128, np=64, nz=64, nrchop=128, npchop=33, nzchop=33, ell=4.0, visc=2.0e-4, is_svv=0)
ADJ_DT, ADJ_STEPS, ADJ_CKPT, ADJ_PERT, ADJ_DIRS, ADJ_H = 2.0e-3, 200, 20, 1.0e-5, 8, 1.0e-6


def adjoint_case(args):
    """The gradient of the final perturbation kinetic energy: Lamb-Oseen vortex of core radius 1
    (the q-vortex recipe with q -> infinity, so chi = 0 before the perturbation), Re = 5000,
    128 x 64 x 64, ELL = 4, dt = 2e-3, 200 steps, checkpoint every 20, seeded perturbation of
    amplitude 1e-5 on |m| <= 4, |k| <= 8, SVV off (the adjoint needs it off).  Reports the adjoint's
    cost against the forward over the same horizon, central differences along 8 seeded unit
    directions (h = 1e-6) in FP64, and the mixed form's J and gradient against FP64's."""
    from mlegs_gb300 import fields, vortex
    from mlegs_gb300.kit import Kit, MIXED, PLAIN_FP64
    from mlegs_gb300.params import make_params
    p = make_params(**ADJ_WORKLOAD)
    kit = Kit(p)
    st = vortex.VortexState(kit)
    pert = (fields.spectral_noise(p, kit.dims, 2001, amp=ADJ_PERT, decay=0.3, m_max=4, k_max=8),
            fields.spectral_noise(p, kit.dims, 2002, amp=ADJ_PERT, decay=0.3, m_max=4, k_max=8))
    vortex.qvort_init(kit, st, q=np.inf, uz_b=0.0, pert=pert)
    psi0, chi0 = st.psi.get(), st.chi.get()

    def ip(a, b):
        return float(np.sum((np.conj(a) * b).real))

    out = {"workload": "Lamb-Oseen NR=128 NP=64 NZ=64 ELL=4 Re=5000 dt=2e-3 200 steps ckpt 20 pert 1e-5 SVV off"}
    for mode, tag in ((PLAIN_FP64, "fp64"), (MIXED, "mixed")):
        kit.set_precision(mode)
        # forward: the same start-up and steps as the adjoint's forward (J only)
        kit.adjoint_run(st.psi, st.chi, st.uz, ADJ_DT, 2, 1)
        kit.sync()
        t0 = time.perf_counter()
        J = kit.adjoint_run(st.psi, st.chi, st.uz, ADJ_DT, ADJ_STEPS, ADJ_CKPT)
        kit.sync()
        t_fwd = time.perf_counter() - t0
        gp, gc = kit.scalar(), kit.scalar()
        kit.adjoint_run(st.psi, st.chi, st.uz, ADJ_DT, 2, 1, gp, gc)
        kit.sync()
        t0 = time.perf_counter()
        Jg = kit.adjoint_run(st.psi, st.chi, st.uz, ADJ_DT, ADJ_STEPS, ADJ_CKPT, gp, gc)
        kit.sync()
        t_adj = time.perf_counter() - t0
        g = (gp.get()[0], gc.get()[0])
        out[tag] = {"J": J, "forward_s": t_fwd, "adjoint_run_s": t_adj,
                    "adjoint_over_forward": t_adj / t_fwd,
                    "sweep_over_forward": (t_adj - t_fwd) / t_fwd,
                    "note": "adjoint_run = forward with checkpoints + backward sweep recomputing each segment"}
        out[tag + "_grad"] = g
        assert Jg == J
    g64, gm = out.pop("fp64_grad"), out.pop("mixed_grad")
    num = np.sqrt(sum(np.sum(np.abs(a - b) ** 2) for a, b in zip(gm, g64)))
    den = np.sqrt(sum(np.sum(np.abs(b) ** 2) for b in g64))
    out["mixed"]["grad_rel_l2_vs_fp64"] = float(num / den)
    out["mixed"]["J_rel_vs_fp64"] = abs(out["mixed"]["J"] - out["fp64"]["J"]) / out["fp64"]["J"]
    # central differences of the FP64 J along seeded unit directions
    kit.set_precision(PLAIN_FP64)
    errs, errs_m = [], []
    for i in range(args.adjoint_dirs):
        dp = fields.spectral_noise(p, kit.dims, 3000 + i, amp=1.0, decay=0.3)
        dc = fields.spectral_noise(p, kit.dims, 4000 + i, amp=1.0, decay=0.3)
        sc = 1.0 / np.sqrt(ip(dp, dp) + ip(dc, dc))
        dp, dc = dp * sc, dc * sc
        Js = []
        for sgn in (1.0, -1.0):
            P = kit.scalar(psi0[0] + sgn * ADJ_H * dp, psi0[1], "FFF")
            C = kit.scalar(chi0[0] + sgn * ADJ_H * dc, chi0[1], "FFF")
            Js.append(kit.adjoint_run(P, C, st.uz, ADJ_DT, ADJ_STEPS, ADJ_CKPT))
            P.free(); C.free()
        fd = (Js[0] - Js[1]) / (2 * ADJ_H)
        an = ip(g64[0], dp) + ip(g64[1], dc)
        am = ip(gm[0], dp) + ip(gm[1], dc)
        errs.append(abs(fd - an) / abs(fd))
        errs_m.append(abs(fd - am) / abs(fd))
    out["fp64"]["fd_directions"] = args.adjoint_dirs
    out["fp64"]["fd_max_rel_err"] = float(max(errs)) if errs else None
    out["fp64"]["fd_h"] = ADJ_H
    out["mixed"]["fd_max_rel_err_vs_fp64_fd"] = float(max(errs_m)) if errs_m else None
    out["mixed"]["note_grad"] = ("the gradient's rel L2 gap to FP64 sits on the last active radial row of each m, a mode "
                                 "unstable with SVV off whose sensitivity magnifies the ~1e-10 trajectory difference; "
                                 "directional derivatives along the FD directions are the fd_max_rel_err_vs_fp64_fd")
    kit.close()
    return out


def run_profile(args):
    """--profile-run: only the set-up and W + K steps of the chosen form (for ncu launch lists)."""
    from mlegs_gb300 import vortex
    from mlegs_gb300.kit import Kit, MIXED, PLAIN_FP64
    p = workload_params()
    kit = Kit(p, precision=PLAIN_FP64 if args.precision == "plain" else MIXED)
    st = vortex.VortexState(kit)
    vortex.qvort_init(kit, st, q=Q, uz_b=0.0, pert=perturbation(p, kit.dims))
    kit.advection_rhs(st.psi, st.chi, st.nlpsi, st.nlchi, st.uz)
    for a, b in (("psi_p", "psi"), ("chi_p", "chi"), ("nlpsi_p", "nlpsi"), ("nlchi_p", "nlchi")):
        getattr(st, a).copy_from(getattr(st, b))
    kit.vortex_run(*st.args(), DT, args.warmup, st.gains)
    l0 = kit.launch_count()
    t0 = time.perf_counter()
    kit.vortex_run(*st.args(), DT, args.steps, st.gains)
    kit.sync()
    dt_s = time.perf_counter() - t0
    print(json.dumps({"profile_run": args.precision, "steps": args.steps, "ms_per_step_wall": 1e3 * dt_s / args.steps,
                      "launches_per_step": (kit.launch_count() - l0) / args.steps}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--accuracy-steps", type=int, default=1000)
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-sweep", action="store_true")
    ap.add_argument("--large", action="store_true", help="also the 512x512x256 case (several minutes)")
    ap.add_argument("--adjoint-dirs", type=int, default=8)
    ap.add_argument("--profile-run", action="store_true")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "plain"])
    args = ap.parse_args()
    if args.profile_run:
        run_profile(args)
        return
    rank, world, local, pg = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world, pg)
    else:
        run_ours(args, rank, world, local, pg)
    if pg:
        pg.barrier()
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
