"""Benchmark of the TTSH3D timestep on GB300: lattice-site-steps per second.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision 32|64] [--workload NAME]

Workload (default "2x256"): the 256^3 droplet case, run as two droplets in one
batch (zeta = 0.005 and 0.02, R = 64, xi = 2, seed 1, reference constants,
reference physics: continuous k^2 and the stale-halo divergence), FP32 fields and
FFT. "1x256" is one droplet (zeta 0.02); "64x128" is the 64-droplet sweep of 128^3
boxes; "24mixed" is 24 droplets of 96/128/160/192^3; "1x512" the single 512^3 droplet.

The metric is Msite*steps/s = (sum over droplets of N^3) * steps / seconds / 1e6,
timed with CUDA events on the library's stream around exactly K steps after W
warm-up steps. The fields (>= 1.2 GB per 256^3 droplet in FP32) are far larger
than L2 (~126 MB), so no L2 flush is needed between steps.

--impl reference times the reference program itself (TTSH3D.cu, patched only in
init/dump/timing, built with its own nvcc line; one 256^3 droplet, FP64, zeta=0,
on the same GPU). If that program is not built, the FP64 C++/OpenMP restatement
of the same step is timed on the host cores instead.

Under torchrun (N > 1) every rank runs its own replica of the workload (the path
has no exchange between droplets): weak scaling, time = max over ranks.
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
for _p in (os.path.join(ROOT, "bacterial-droplet_gb300"), os.path.join(ROOT, "oracle"),
           os.path.join(ROOT, "tests", "golden")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "Msite·steps/s at 256³, batched FP32 vs plain FP64 on one GB300; %HBM peak"
UNIT = "Msite*steps/s"
# B_alg: the compulsory traffic of the minimal three-phase schedule, 34 words per site-step
# (136 B in FP32, 272 B in FP64): the RHS reads phi, P, u (7) and writes phi', u*, P* and the
# two Poisson sources (9); the FFT moves each source once (2 + 2); the correction reads u*, P*,
# the two pressures (8) and writes u, P (6). The %HBM of a step uses B_alg.
# KERNEL_WORDS: the algorithmic words of each kernel of this build (the divergence and every FFT
# pass are separate launches here), used for the per-kernel roofline.
B_ALG_WORDS = 34
KERNEL_WORDS = {
    # the fused form stores u, u*, P* compensated (FP32 + a bf16 remainder: half a word each)
    "fused_rhs": 20.5,      # reads phi, P, u (7), the compensations of phi, u (1 + 1.5); writes phi',
                            # u*, P* (7) and their compensations (1 + 3)
    "fused_div": 11,        # reads u*, P* and their compensations (6 + 3); writes the packed source W (2)
    "fused_correct": 18.5,  # reads u*, P*, compensations, the packed pressure (6 + 3 + 2); writes u, P and
                            # the compensation of u (6 + 1.5)
    "stage1": 17, "stage2": 27, "div": 8, "correct": 14,  # plain form
    "fft_x_fwd": 4, "fft_y_fwd": 4, "fft_z_poisson": 4, "fft_y_inv": 4, "fft_x_inv": 4,
    "fft_xy_fwd": 4, "fft_yx_inv": 4,  # x and y of a plane in one launch: W read and written once
}

# DRAM bytes per site of the dominant FP32 kernels, dram__bytes_read.sum + dram__bytes_write.sum
# of one ncu capture of the default configuration on a 256^3 droplet (--clock-control none); a
# launch over more sites scales with the sites (every kernel streams its planes once).
TRAFFIC_BYTES_PER_SITE_F32 = {
    "fused_rhs": (1061.009e6 + 710.105e6) / 256 ** 3,
}
# Warp instructions per site of the dominant FP32 kernels (smsp__inst_executed.sum of the same
# capture / sites): with the SM count, 4 schedulers per SM and the sampled SM clock they give the
# time the kernel's instruction issue alone takes, the other bound of an on-chip-limited kernel.
INSTR_PER_SITE_F32 = {
    "fused_rhs": 539993606 / 256 ** 3,
}


def workload(name: str):
    """List of droplets: (N, R, xi, seed, zeta)."""
    if name == "2x256":
        return [(256, 64.0, 2.0, 1, 0.005), (256, 64.0, 2.0, 1, 0.02)]
    if name == "1x256":
        return [(256, 64.0, 2.0, 1, 0.02)]
    if name == "64x128":
        rng = np.random.default_rng(2024)
        R = rng.uniform(20, 40, 64)
        z = np.exp(rng.uniform(np.log(1e-3), np.log(5e-2), 64))
        return [(128, float(R[i]), 2.0, 100 + i, float(z[i])) for i in range(64)]
    if name == "24mixed":
        out = []
        for k, L in enumerate((96, 128, 160, 192)):
            for j in range(6):
                i = 6 * k + j
                out.append((L, 0.3 * L, 2.0, 200 + i, 0.01 if i % 2 == 0 else 0.03))
        return out
    if name == "1x512":
        return [(512, 160.0, 3.0, 7, 0.02)]
    if name == "1x128":
        return [(128, 32.0, 2.0, 1, 0.02)]
    if name == "1x64":
        return [(64, 16.0, 2.0, 0, 0.01)]
    raise SystemExit("unknown workload " + name)


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        os.unlink(self.path)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            if len(r) >= 9:
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            return float(json.load(open(p))["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def make_sim(ttsh, drops, precision, k2_mode=0, quirks=1, form=0):
    inps, exts = [], []
    for (N, R, xi, seed, zeta) in drops:
        inps.append(ttsh.default_input(Nx=N, Ny=N, Nz=N))
        exts.append(ttsh.default_ext(precision=precision, zeta=zeta, R=R, xi=xi, seed=seed, k2_mode=k2_mode,
                                     quirks=quirks, form=form))
    return ttsh.Sim(inps, exts, device=0)


def init_states(ttsh, drops, pinned: bool):
    import torch
    states = []
    cache = {}
    for (N, R, xi, seed, zeta) in drops:
        key = (N, R, xi, seed)
        if key not in cache:
            phi, P = ttsh.init_droplet(N, R, xi, seed)
            if pinned:
                tp = torch.empty((N, N, N), dtype=torch.float64, pin_memory=True)
                tq = torch.empty((3, N, N, N), dtype=torch.float64, pin_memory=True)
                tu = torch.zeros((3, N, N, N), dtype=torch.float64, pin_memory=True)
                tp.numpy()[:] = phi
                tq.numpy()[:] = P
                cache[key] = (tp.numpy(), tq.numpy(), tu.numpy(), (tp, tq, tu))
            else:
                cache[key] = (phi, P, np.zeros((3, N, N, N)), None)
        states.append(cache[key])
    return states


def cpu_baseline_sample():
    """The FP64 oracle (C++/OpenMP restatement) on one 256^3 droplet for 2 steps, host cores."""
    import oracle
    oracle.build()
    n = oracle.set_threads(os.cpu_count() or 1)
    N, steps = 256, 2
    phi, P = oracle.init_droplet(N, 64.0, 2.0, 1)
    s = oracle.new_state(N)
    s["phi"][:] = phi
    s["px"][:], s["py"][:], s["pz"][:] = P
    t0 = time.perf_counter()
    oracle.step(s, steps, N, zeta=0.005)
    dt = time.perf_counter() - t0
    return {"value": N ** 3 * steps / dt / 1e6, "unit": UNIT, "cores": n, "kind": "port",
            "sample": "FP64 C++/OpenMP restatement of the step, one 256^3 droplet (zeta=0.005), %d steps, %.1f s"
                      % (steps, dt)}


def run_reference(args):
    """--impl reference: the reference program on the GPU, else the oracle port on the host."""
    out = {"metric": METRIC, "unit": UNIT, "impl": "reference", "higher_is_better": True, "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "scaling": "weak", "vs_baseline": None, "data": "synthetic"}
    binary = None
    try:
        import make_ref
        binary = make_ref.build()
    except Exception as e:  # report and fall back
        out["note"] = "reference program not built: %s" % str(e)[:200]
    if binary:
        # the reference program runs on with failing CUDA calls when no GPU is visible (and then
        # times nothing): only run it where one is
        import torch
        if not torch.cuda.is_available():
            out["note"] = "no GPU visible: the reference program cannot run here"
            binary = None
    if binary:
        # nothing of libttsh is loaded here: the input file is written in Python and the initial
        # fields come from the oracle's restatement of the droplet construction (same bits)
        import make_ref_golden as G
        import oracle
        N = 256
        phi, P = oracle.init_droplet(N, 64.0, 2.0, 1)
        st = {k: np.zeros((N, N, N)) for k in G.FIELDS}
        st["phi"] = phi
        st["px"], st["py"], st["pz"] = P
        try:
            with tempfile.TemporaryDirectory() as d:
                t0 = time.perf_counter()
                log = G.run_reference(binary, d, N, st, Ts=(args.warmup + args.steps - 0.5) * 0.002, dte=1e9,
                                      expo=0, warmup=args.warmup, nfields=7)
                wall = time.perf_counter() - t0
            line = [l for l in log.splitlines() if l.startswith("TTSH_REF_TIMING")][-1]
            kv = dict(x.split("=") for x in line.split()[1:])
            steps, sec = int(kv["steps"]), float(kv["seconds"])
        except Exception as e:  # e.g. no GPU visible: report it and time the oracle port instead
            out["note"] = "reference program failed: %s" % str(e)[:300]
            binary = None
    if binary:
        v = N ** 3 * steps / sec / 1e6
        out.update(value=v, ms_per_step=1e3 * sec / steps, dtype="f64",
                   config={"workload": "1 droplet x 256^3 (R=64, xi=2, seed 1, zeta=0: the reference has no "
                                       "active stress), reference program TTSH3D.cu on the GPU",
                           "build": "nvcc -std=c++14 --cudart=shared -lcufft (run_cuda.pl:4), no -arch",
                           "timing": "cudaDeviceSynchronize + steady_clock around the step loop after warm-up",
                           "process_wall_s": round(wall, 1)},
                   cpu_baseline={"value": v, "unit": UNIT, "cores": 0, "kind": "reference",
                                 "sample": "the reference program's own step loop on the GPU (it has no CPU "
                                           "path), %d steps at 256^3" % steps},
                   e2e={"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0})
    else:
        cb = cpu_baseline_sample()
        out.update(value=cb["value"], dtype="f64", config={"workload": "oracle port, " + cb["sample"]},
                   cpu_baseline=cb, e2e={"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                                         "d2h_bytes_per_step": 0})
    print(json.dumps(out))


def run_snapshot(args):
    """--snapshot: the snapshot writer (conf_<te>.dat, ExpoConf's text layout) in text bytes per
    second at N^3, ours (synchronous ttsh_write_conf, and ttsh_write_conf_async issued before K
    steps: the host time it takes and how much of its formatting the steps hide) against the
    reference program's own ExpoConf (TTSH3D.cu:899-1014: 58 device-to-host copies, then one line
    per site through ofstream with endl). The reference's time is the difference of two runs of
    its timed step loop (warm-up 1, steps 2-4): one with a snapshot at step 3, one without."""
    import shutil
    import ttsh
    N, K = args.snapshot_n, args.steps
    out = {"metric": "snapshot text bytes/s", "unit": "MB/s", "n": N, "impl": "snapshot"}
    base = tempfile.mkdtemp(prefix="ttsh_conf_")
    try:
        free = shutil.disk_usage(base).free
        need = 3 * 125 * N ** 3 + 15 * 8 * N ** 3
        if free < need:
            raise SystemExit("snapshot bench: %d bytes free under %s, %d needed" % (free, base, need))
        phi, P = ttsh.init_droplet(N, N / 4.0, 2.0, 1)
        inp = ttsh.default_input(Nx=N, Ny=N, Nz=N)
        with ttsh.Sim(inp, ttsh.default_ext(precision=32, zeta=0.02, form=ttsh.FORM_FUSED)) as s:
            s.set_state(0, phi, P, np.zeros_like(P))
            s.step(3)
            s.sync()
            path = os.path.join(base, "conf_1.dat")
            t0 = time.perf_counter()
            s.write_conf(0, path)
            t1 = time.perf_counter()
            nbytes = os.path.getsize(path)
            os.remove(path)
            s.sync()
            t2 = time.perf_counter()
            s.step(K)
            s.sync()
            t3 = time.perf_counter()
            s.write_conf_async(0, path)
            t4 = time.perf_counter()
            s.step(K)
            s.sync()
            t5 = time.perf_counter()
            s.conf_wait()
            t6 = time.perf_counter()
            nbytes_async = os.path.getsize(path)  # a later state: the signs, so the length, differ
            os.remove(path)
        out["ours"] = {"bytes": nbytes, "sync_s": t1 - t0, "sync_MBps": nbytes / (t1 - t0) / 1e6,
                       "steps": K, "steps_alone_s": t3 - t2, "async_call_s": t4 - t3,
                       "steps_after_async_s": t5 - t3, "async_total_s": t6 - t3, "async_bytes": nbytes_async,
                       "exposed_s": (t6 - t3) - (t3 - t2),
                       "form": "FP32 fused, 1 droplet, cores %d" % (os.cpu_count() or 0)}
        binary = None
        if args.snapshot_skip_reference:
            out["reference"] = {"skipped": "--snapshot-skip-reference"}
        else:
            try:
                import make_ref
                binary = make_ref.build()
            except Exception as e:
                out["reference"] = {"unavailable": "reference program not built: %s" % str(e)[:200]}
        if binary:
            import make_ref_golden as G
            import oracle
            phi, P = oracle.init_droplet(N, N / 4.0, 2.0, 1)
            st = {k: np.zeros((N, N, N)) for k in G.FIELDS}
            st["phi"] = phi
            st["px"], st["py"], st["pz"] = P
            dt, T0 = 0.002, 1e-6
            secs, sizes = [], []
            for dte in (1e9, 2.5 * dt):  # no snapshot / one at step 3 (T = 3 dt + T0)
                d = os.path.join(base, "ref_%g" % dte)
                log = G.run_reference(binary, d, N, st, Ts=3.5 * dt, dte=dte, expo=1, warmup=1, nfields=7, T0=T0)
                line = [l for l in log.splitlines() if l.startswith("TTSH_REF_TIMING")][-1]
                kv = dict(x.split("=") for x in line.split()[1:])
                secs.append(float(kv["seconds"]))
                confs = [f for f in os.listdir(os.path.join(d, "data_1")) if f.startswith("conf_")]
                sizes.append(sum(os.path.getsize(os.path.join(d, "data_1", f)) for f in confs))
                shutil.rmtree(d, ignore_errors=True)
            expo_s = secs[1] - secs[0]
            out["reference"] = {"bytes": sizes[1], "loop_s_without": secs[0], "loop_s_with": secs[1],
                                "expoconf_s": expo_s, "MBps": sizes[1] / expo_s / 1e6 if expo_s > 0 else None}
            if out["reference"]["MBps"]:
                out["sync_speedup"] = out["ours"]["sync_MBps"] / out["reference"]["MBps"]
    finally:
        shutil.rmtree(base, ignore_errors=True)
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", type=int, default=32, choices=[32, 64])
    ap.add_argument("--workload", default="2x256")
    ap.add_argument("--k2", type=int, default=0, choices=[0, 1])
    ap.add_argument("--form", type=int, default=0, choices=[0, 1, 2], help="0 auto, 1 plain, 2 fused")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 one-droplet reference point")
    ap.add_argument("--no-tune", action="store_true", help="keep the default kernel configuration")
    ap.add_argument("--snapshot", action="store_true",
                    help="measure the snapshot writer (text bytes/s) against the reference's ExpoConf and exit")
    ap.add_argument("--snapshot-n", type=int, default=256)
    ap.add_argument("--snapshot-skip-reference", action="store_true",
                    help="with --snapshot: time only this library's writer")
    args = ap.parse_args()
    if args.snapshot:
        run_snapshot(args)
        return
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")

    from ttsh import replicas
    rank, world, local = replicas.env_rank()

    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import ttsh

    drops = workload(args.workload)
    sites = sum(d[0] ** 3 for d in drops)
    sim = make_sim(ttsh, drops, args.precision, k2_mode=args.k2, form=args.form)
    # one non-default stream shared by the library and the timing events
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sim.set_stream(stream.cuda_stream)
    states = init_states(ttsh, drops, pinned=False)
    for i, (phi, P, u, _) in enumerate(states):
        sim.set_state(i, phi, P, u)
    # kernel configuration per droplet size (FFT kind / lines / radix order, z-planes per CTA of
    # the fused kernels), timed on these fields before the warm-up
    tuning = None if args.no_tune else sim.autotune()
    sim.step(args.warmup)
    torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    sim.step(args.steps)
    ev1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    ms = replicas.max_over_ranks(ev0.elapsed_time(ev1), device="cuda")
    value = sites * world * args.steps / (ms / 1e3) / 1e6
    stats = [sim.reduce(i, check=False) for i in range(len(drops))]

    # per-kernel device times (events around each launch on the library's stream)
    prof = sim.profile_kernels(20)
    torch.cuda.synchronize()
    wbytes = 4 if args.precision == 32 else 8
    peak, peak_kind = measured_peak_hbm()
    dom = max(prof.items(), key=lambda kv: kv[1][0])
    dom_name, (dom_ms, dom_launches) = dom
    dom_bytes = KERNEL_WORDS.get(dom_name, 0) * wbytes * sites
    achieved = dom_bytes / (dom_ms / 1e3) / 1e9 if dom_ms > 0 else 0.0
    traffic = None
    if args.precision == 32 and dom_name in TRAFFIC_BYTES_PER_SITE_F32:
        traffic = TRAFFIC_BYTES_PER_SITE_F32[dom_name] * sites
    launches = sim.launches_per_step()
    issue_ms = None
    if args.precision == 32 and dom_name in INSTR_PER_SITE_F32:
        sm_mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz")
        if sm_mhz:
            sms = torch.cuda.get_device_properties(local).multi_processor_count
            issue_ms = INSTR_PER_SITE_F32[dom_name] * sites / (sms * 4 * sm_mhz * 1e6) * 1e3

    # end to end through the public API: host state -> device, K steps each followed by the
    # FP64 mass/divergence read-back, final state -> host
    e2e = None
    if not args.no_e2e:
        pin = init_states(ttsh, drops, pinned=True)
        # pinned host buffers for the final state, as for the initial one
        keep = [(torch.empty((N, N, N), dtype=torch.float64, pin_memory=True),
                 torch.empty((3, N, N, N), dtype=torch.float64, pin_memory=True),
                 torch.empty((3, N, N, N), dtype=torch.float64, pin_memory=True)) for (N, *_r) in drops]
        outs = [tuple(t.numpy() for t in k) for k in keep]
        # one pinned row of diagnostics partials per step, filled asynchronously
        diag = torch.empty((args.steps, sim.partials_size()), dtype=torch.float64, pin_memory=True).numpy()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        esampler = ClockSampler(local)
        esampler.start()
        t0 = time.perf_counter()
        for i, (phi, P, u, _) in enumerate(pin):
            sim.set_state(i, phi, P, u)
        t1 = time.perf_counter()
        for k in range(args.steps):
            sim.step(1)
            sim.reduce_all_async(diag[k], mass_only=True)
        t2 = time.perf_counter()
        for i, (phi, P, u) in enumerate(outs):
            lib_rc = ttsh.lib().ttsh_get_state(sim.handle, i, ttsh._p(phi), ttsh._p(P), ttsh._p(u), None, None)
            ttsh._check(lib_rc)
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        eclocks = esampler.stop()
        last = sim.stats_from_partials(diag[args.steps - 1], check=False)
        assert last[0]["steps"] == diag[0, 0] + args.steps - 1 and all(d["nonfinite"] == 0 for d in last)
        wall = replicas.max_over_ranks(t3 - t0, device="cuda")
        split = {"set_state_s": t1 - t0, "steps_s": t2 - t1, "get_state_s": t3 - t2}
        h2d = sum(7 * d[0] ** 3 * 8 for d in drops)
        d2h = args.steps * 8 * (diag.shape[1] - 2 - len(drops)) + sum(7 * d[0] ** 3 * 8 for d in drops)  # partials + state
        e2e = {"value": sites * world * args.steps / wall / 1e6, "unit": UNIT,
               "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
               "note": "public API (ttsh.Sim): set_state from pinned host FP64 arrays, %d x (step + FP64 "
                       "mass diagnostics of every droplet, ttsh_reduce_all_async into pinned host rows, read after the "
                       "final sync), get_state of all fields into "
                       "pinned host FP64 arrays; wall clock" % args.steps, "split": split,
               "clocks": eclocks}

    # the other side of the metric: the plain FP64 form, one 256^3 droplet per launch (R = 64,
    # xi = 2, seed 1, zeta = 0.02), on the same GPU in the same run, CUDA events around its steps
    fp64 = None
    if not args.no_fp64 and args.precision == 32:
        k64 = max(3, min(args.steps, 10))
        with make_sim(ttsh, [(256, 64.0, 2.0, 1, 0.02)], 64, k2_mode=args.k2, form=1) as s64:
            s64.set_stream(stream.cuda_stream)
            phi, P, u, _ = init_states(ttsh, [(256, 64.0, 2.0, 1, 0.02)], pinned=False)[0]
            s64.set_state(0, phi, P, u)
            s64.step(3)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            s64.step(k64)
            b.record(stream)
            torch.cuda.synchronize()
            ms64 = replicas.max_over_ranks(a.elapsed_time(b), device="cuda")
        v64 = 256 ** 3 * world * k64 / (ms64 / 1e3) / 1e6
        fp64 = {"value": v64, "unit": UNIT, "ms_per_step": ms64 / k64, "steps": k64, "warmup": 3,
                "workload": "1 x 256^3 (R=64, xi=2, seed 1, zeta=0.02), FP64 plain form (one droplet per launch, "
                            "the reference's arithmetic order), same GPU and run",
                "ratio_fp32_batched_over_fp64_plain": value / v64}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline_sample()

    if rank == 0:
        hbm_frac = value * 1e6 * B_ALG_WORDS * wbytes / (peak * 1e9)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if args.precision == 32 else "f64", "data": "synthetic",
            "config": {"workload": args.workload + ": " + ", ".join(
                "%d^3 (R=%g, xi=%g, seed %d, zeta=%g)" % d for d in drops[:4]) + (" ..." if len(drops) > 4 else ""),
                "droplets": len(drops), "sites_per_gpu": sites, "form": "fused" if "fused_rhs" in prof else "plain",
                "physics": "reference (continuous k^2, stale-halo divergence)" if args.k2 == 0 else "discrete k^2",
                "l2": "inputs larger than L2 (%.1f GB of fields per GPU)" % (sites * 22 * wbytes / 1e9),
                "parallelism": "replicas" if world > 1 else "1 GPU",
                "tuning": "default" if tuning is None else [
                    "N=%d x%d: fft %s, zc %s" % (t["N"], t["n"], {0: "register per axis", 2: "register x+y per plane"}.get(
                        t["fft_kind"], "stockham lb=%d radix=%s" % (t["fft_lb"], t["radix"])), t["zc"])
                    for t in tuning]},
            "hbm_pct_of_step": 100 * hbm_frac,
            "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "traffic_source": "ncu DRAM read+write bytes of one 256^3 launch, scaled by sites"
                         if traffic is not None else None,
                         "peak_kind": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else
                         peak_kind, "bytes_per_launch": dom_bytes, "ms_per_launch": dom_ms / max(1, dom_launches),
                         "issue_bound_ms": issue_ms,
                         "issue_frac": issue_ms / (dom_ms / max(1, dom_launches)) if issue_ms and dom_ms > 0 else None,
                         "issue_source": "ncu warp instructions per site of one 256^3 launch x sites / (SMs x 4 "
                                         "schedulers x median SM clock under load)" if issue_ms else None},
            "kernels_ms_per_step": {k: round(v[0], 4) for k, v in prof.items()},
            "gpu_launches": launches * args.steps,
            "launches_per_step": launches,
            "clocks": clocks,
            "mass": [s["mass"] for s in stats],
            "max_div_u": [s["max_div_u"] for s in stats],
        }
        if e2e:
            line["e2e"] = e2e
        if fp64:
            line["fp64_plain"] = fp64
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line))
    sim.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
