"""Benchmark of the GB300 walker path: plain CPMG at scale, walker-steps/s.

Workload (one "step" = one full CPMG walk over the synthetic input):
  cpmg-2phase-400: 400^3 uint8 label image (0 = pore, 1/2 = solid phase A/B), overlapping spheres
  of radius 6-20 voxels labelled A or B with p = 0.5 until porosity <= 0.25 (seed 2); 1,000,000
  walkers placed uniformly in pore voxels (SEED 7); rho_A = 5, rho_B = 25 um/s; D0 = 2.5 um^2/ms;
  echo time 0.1 ms = 1 walk step at voxel size sqrt(6 D0 te) = 1.2247 um; 20,000 echoes; noflux.
  2e10 walker-steps per step. Synthetic data (the reference ships no benchmark images).

Reported:
  value      walker-steps/s of the walk kernels with all inputs resident in HBM (CUDA events on the
             engine's stream; L2 flushed before every timed step by writing a 512 MB buffer)
  e2e        the same metric through the C ABI from pinned host buffers: image labels and walker
             initial state copied host->device, echo train and per-echo collisions copied back
  roofline   the instruction-issue bound that binds: algorithmic warp-instructions (48 int32 slots =
             1.5 per walker-step) per launch / launch time, against SMs x 4 schedulers x the sampled
             SM clock; the kernel's measured instruction count (ncu) beside it; the gathered bytes
             against the HBM copy peak as a secondary entry
  cpu_baseline  the oracle's CPU walk (port of the reference's Walker::walk) on a bounded walker
             sample with all host threads
  rho_fit_batch  (default workload) GPU-seconds of the batched relaxivity fit over 64 uneven images
             against per-image plain CPMG + the restated GA, the GA run on every image

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--workload NAME]
  workloads: cpmg-2phase-400 (default), cpmg-1phase-100, cpmg-2phase-small, map-400, pfgse-256[-small],
             rho-fit-multiphase[-small], rho-fit-batch[-small]
"""
from __future__ import annotations

import argparse
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

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


def workload(name: str):
    if name == "map-400":
        # the reference's collision-mapping walk (mapSimulation) on the headline image and walkers:
        # 20,000 steps, per-walker collision counts out
        w = workload("cpmg-2phase-400")
        w.update(name=name, map=True)
        return w
    if name == "cpmg-2phase-400":
        return dict(name=name, shape=(400, 400, 400), rmin=6.0, rmax=20.0, porosity=0.25, n_phases=2, img_seed=2,
                    walkers=1_000_000, seed=7, rho=[5.0, 25.0], d0=2.5, te=0.1, echoes=20_000, bc="noflux")
    if name == "cpmg-1phase-100":
        return dict(name=name, shape=(100, 100, 100), rmin=4.0, rmax=10.0, porosity=0.30, n_phases=1, img_seed=1,
                    walkers=10_000, seed=7, rho=[10.0], d0=2.5, te=0.2, echoes=2_000, bc="noflux", res=1.0)
    if name in ("cpmg-field-400", "cpmg-field-small"):
        # the headline image and walkers in a uniform internal field of 1 T/m along z (RESIDUAL_FIELD:
        # uniform), te = 2 steps (one step per inversion), gyromagnetic ratio 42.576 MHz/T
        return dict(name=name, shape=(400, 400, 400), rmin=6.0, rmax=20.0, porosity=0.25, n_phases=2, img_seed=2,
                    walkers=1_000_000, seed=7, rho=[5.0, 25.0], d0=2.5, te=0.2, res=1.224744871391589,
                    echoes=10_000 if name == "cpmg-field-400" else 100, bc="noflux", field=(1.0, 2))
    if name == "cpmg-2phase-small":  # profiling case: same kernel, smaller walk
        return dict(name=name, shape=(400, 400, 400), rmin=6.0, rmax=20.0, porosity=0.25, n_phases=2, img_seed=2,
                    walkers=1_000_000, seed=7, rho=[5.0, 25.0], d0=2.5, te=0.1, echoes=200, bc="noflux")
    raise SystemExit(f"unknown workload {name}")


def derived(w):
    res = w.get("res", float(np.sqrt(6.0 * w["d0"] * w["te"])))  # dt = res^2 / (6 D0) = te
    dt = res * res / (6.0 * w["d0"])
    spe = max(1, int(round(w["te"] / dt)))
    f = 1.0 - (2.0 / 3.0) * (np.asarray(w["rho"], np.float64) * res) / (w["d0"] * 1e3)
    return res, spe, f


def build_inputs(w):
    from randomwalk_nmr_gb300 import host

    labels, por = host.synth_spheres(w["shape"], w["rmin"], w["rmax"], w["porosity"], w["n_phases"], seed=w["img_seed"])
    blocks, _ = host.pack_blocks(labels)
    x, y, z, s, info = host.place_walkers(blocks, labels.shape, w["walkers"], w["seed"])
    return labels, por, (x, y, z, s)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.out = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.out.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(PEAKS_FILE) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured", p
    except Exception:
        return FALLBACK_HBM_GBS, "fallback", {}


# Algorithmic integer work of one walker step, in 32-thread warp-instructions: about 48 int32
# issue slots (xorshift64 ~12, mod 6 ~8, move and border select ~8, block and bit index ~12, bit
# test ~4, collision count and position select ~4), i.e. 1.5 warp-instructions per walker-step.
ALG_WARP_INST_PER_STEP = 48 / 32


def kernel_counters(name):
    """ncu counters of a workload's walk kernel, committed beside its profile summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "kernel_counters.json")) as fh:
            return json.load(fh).get(name, {})
    except Exception:
        return {}


def issue_roofline(rate, steps_per_launch, launch_s, device, clocks, peaks, counters):
    """Instruction-issue roofline of the walk kernel, the bound that binds: achieved = algorithmic
    warp-instructions per launch / the launch's average device time; peak = SMs (from the device) x 4
    warp schedulers x the SM clock sampled during the timed region (one warp-instruction each per
    cycle). The measured instruction count of the kernel (an ncu capture) is reported beside it."""
    import torch

    sms = torch.cuda.get_device_properties(device).multi_processor_count
    mhz = float(clocks.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0))
    peak = sms * 4 * mhz * 1e6 / 1e9
    achieved = ALG_WARP_INST_PER_STEP * steps_per_launch / launch_s / 1e9
    out = {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "Gwarp-inst/s", "frac": achieved / peak,
           "traffic": counters.get("dram_bytes_per_launch"), "traffic_unit": "DRAM bytes per launch (ncu)",
           "alg_warp_inst_per_walker_step": ALG_WARP_INST_PER_STEP, "walker_steps_per_launch": steps_per_launch,
           "launch_ms": launch_s * 1e3, "sm_count": sms, "sm_mhz": mhz,
           "peak_source": "SM count (cudaDevAttrMultiProcessorCount) x 4 schedulers x median sampled SM clock"}
    if counters.get("warp_inst_per_walker_step"):
        inst = counters["warp_inst_per_walker_step"]
        out["measured"] = {"warp_inst_per_walker_step": inst, "issue_active_pct": counters.get("issue_active_pct"),
                           "l1_hit_pct": counters.get("l1_hit_pct"),
                           "frac_of_issue_peak": inst * rate / 1e9 / peak,
                           "source": "ncu smsp__inst_executed.sum, " + counters.get("source", "profiles/") +
                                     (", " + counters["date"] if counters.get("date") else "")}
    return out


def cpu_baseline(labels, n_phases, walkers, spe, echoes, f, bc, target_s=15.0):
    """The oracle port of the reference's CPU walk on a bounded walker sample, all host threads."""
    from oracle.pyoracle import Oracle, build

    build(with_ref=False)
    o = Oracle()
    threads = os.cpu_count() or 1
    x, y, z, s = walkers
    # calibrate on a small sample, then size the timed sample to ~target_s; the first call packs the
    # image, which the oracle keeps for the later calls, so neither timed call includes it
    n0 = min(len(x), 256 * threads)
    e0 = min(echoes, 2000)
    small = (x[:n0], y[:n0], z[:n0], s[:n0])
    o.cpmg(labels, small, 1, spe, f, bc=bc, n_phases=n_phases, threads=threads)
    t0 = time.perf_counter()
    o.cpmg(labels, small, e0, spe, f, bc=bc, n_phases=n_phases, threads=threads)
    rate = n0 * e0 * spe / max(time.perf_counter() - t0, 1e-3)
    n = int(max(threads * 4, min(len(x), rate * target_s / (echoes * spe))))
    sample = (x[:n], y[:n], z[:n], s[:n])
    t0 = time.perf_counter()
    out = o.cpmg(labels, sample, echoes, spe, f, bc=bc, n_phases=n_phases, threads=threads)
    dt = time.perf_counter() - t0
    return dict(value=n * echoes * spe / dt, unit="walker-steps/s", cores=threads, kind="port",
                sample=f"first {n} of {len(x)} walkers, all {echoes} echoes x {spe} steps ({dt:.1f} s)"), out, sample


def oracle_inputs(w):
    """The workload's image and walkers from the oracle's own restatements of the sphere-pack
    generator and of the reference's random placement: the reference arm loads no product code."""
    from oracle.pyoracle import Oracle, build

    build(with_ref=False)
    o = Oracle()
    labels, por = o.synth_spheres(w["shape"], w["rmin"], w["rmax"], w["porosity"], w["n_phases"], w["img_seed"])
    x, y, z, s, _ = o.place_walkers(labels, w["walkers"], w["seed"])
    return o, labels, por, (x, y, z, s)


def serial_reference_timing(o, labels, walkers, n_phases, spe, echoes, f, bc, target_s=5.0):
    """The reference's own CPU order (NMR_cpmg::image_simulation_omp is serial: its OpenMP pragmas are
    commented out, NMR_cpmg.cpp:209,220) on one core: the oracle's walk with one thread on a walker
    sample sized to about target_s seconds."""
    x, y, z, s = walkers
    n0 = min(len(x), 64)
    e0 = min(echoes, 2000)
    o.cpmg(labels, (x[:1], y[:1], z[:1], s[:1]), 1, spe, f, bc=bc, n_phases=n_phases, threads=1)  # packs the image
    t0 = time.perf_counter()
    o.cpmg(labels, (x[:n0], y[:n0], z[:n0], s[:n0]), e0, spe, f, bc=bc, n_phases=n_phases, threads=1)
    rate = n0 * e0 * spe / max(time.perf_counter() - t0, 1e-3)
    n = int(max(8, min(len(x), rate * target_s / (echoes * spe))))
    t0 = time.perf_counter()
    o.cpmg(labels, (x[:n], y[:n], z[:n], s[:n]), echoes, spe, f, bc=bc, n_phases=n_phases, threads=1)
    dt = time.perf_counter() - t0
    return dict(value=n * echoes * spe / dt, unit="walker-steps/s", cores=1, kind="port",
                sample=f"first {n} of {len(x)} walkers, all {echoes} echoes x {spe} steps, one thread ({dt:.1f} s)")


def run_reference(args, w):
    """Reference arm: the reference's CPU walk (oracle port on the GPU machine) on a bounded sample, its
    inputs from the oracle's own generator and placement (no product code is loaded)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    res, spe, f = derived(w)
    o, labels, por, walkers = oracle_inputs(w)
    threads = os.cpu_count() or 1
    x, y, z, s = walkers
    n = int(os.environ.get("RWNMR_REF_SAMPLE", "0")) or min(len(x), 8 * threads * 64)
    sample = (x[:n], y[:n], z[:n], s[:n])
    echoes = w["echoes"]
    for _ in range(args.warmup):
        o.cpmg(labels, sample, min(echoes, 200), spe, f, bc=w["bc"], n_phases=w["n_phases"], threads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o.cpmg(labels, sample, echoes, spe, f, bc=w["bc"], n_phases=w["n_phases"], threads=threads)
        times.append(time.perf_counter() - t0)
    per = statistics.mean(times)
    value = n * echoes * spe / per
    serial = serial_reference_timing(o, labels, walkers, w["n_phases"], spe, echoes, f, w["bc"])
    line = {"metric": "walker-steps/s (plain CPMG)", "value": value, "unit": "walker-steps/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": per * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32+u64 walk, f64 energy",
            "data": "synthetic", "config": {"workload": w["name"], "walkers_timed": n, "echoes": echoes,
                                            "steps_per_echo": spe},
            "cpu_baseline": {"value": value, "unit": "walker-steps/s", "cores": threads, "kind": "port",
                             "sample": f"first {n} of {len(x)} walkers, all {echoes} echoes per step",
                             "serial": serial},
            "e2e": {"value": value, "unit": "walker-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def _sphere_image(args):
    from randomwalk_nmr_gb300 import host

    shape, rmin, rmax, por, phases, seed, walkers, wseed = args
    lab, p = host.synth_spheres(shape, rmin, rmax, por, phases, seed=seed)
    blocks, _ = host.pack_blocks(lab)
    w = host.place_walkers(blocks, lab.shape, walkers, wseed)[:4]
    return lab, blocks, w, p


def run_fit_multiphase(args):
    print(json.dumps(fit_multiphase(args, args.workload.endswith("-small"), args.workload)))


def fit_multiphase(args, small, name):
    """Differentiable CPMG fit of a multi-phase image: 200^3, 4 solid phases, 500k walkers, 5000 echoes
    of 3 steps; L-BFGS with gradients from the walk's forward sensitivities (one walk per evaluation) vs the
    restated GA (population 64) on the same GPU walk. Returns the result line."""
    import torch

    from randomwalk_nmr_gb300 import Engine
    from randomwalk_nmr_gb300.autograd import cpmg_decay
    from randomwalk_nmr_gb300.fit import fit_rho_adjoint
    from randomwalk_nmr_gb300.ga import GeneticAlgorithm, misfit_fitness

    n, echoes, edge = (50_000, 500, 100) if small else (500_000, 5000, 200)
    lab, blocks, w, por = _sphere_image(((edge, edge, edge), 5.0, 12.0, 0.30, 4, 4, n, 7))
    eng = Engine(0)
    eng.upload_labels(lab, 4)
    eng.upload_walkers(*w)
    rng = np.random.default_rng(5)
    hidden = rng.uniform(2.0, 40.0, 4)
    t2b, spe = 2000.0, 3
    with torch.no_grad():
        clean = cpmg_decay(torch.tensor(hidden), torch.tensor(t2b), eng, echoes, spe).numpy()
    target = clean + rng.normal(0.0, 1e-3, clean.shape)
    res = fit_rho_adjoint(eng, target, np.full(4, 20.0), echoes, spe, t2b, max_evals=args.fit_evals)

    def model(g):
        with torch.no_grad():
            m = cpmg_decay(torch.tensor(np.asarray(g)), torch.tensor(t2b), eng, echoes, spe).numpy()
        ga_gpu[0] += eng.last_kernel_ms * 1e-3
        return m

    ga_gpu = [0.0]
    t0 = time.perf_counter()
    ga = GeneticAlgorithm(misfit_fitness(model, target, 1e-3), [2.0] * 4, [40.0] * 4, population=64, seed=11)
    ga.run(args.ga_generations)
    ga_wall = time.perf_counter() - t0
    # both fits' misfits on one scale: sum ((M - target) / max|target|)^2, the gradient fit's loss,
    # beside the noise floor of the target itself (the misfit of the clean train at the hidden rho)
    scale = float(np.abs(target).max())
    ga_gpu_fit = ga_gpu[0]
    ga_loss = float(np.sum(((model(ga.best[0]) - target) / scale) ** 2))
    floor = float(np.sum(((clean - target) / scale) ** 2))
    line = {"metric": "GPU-seconds of the relaxivity fit (multi-phase CPMG)", "value": res["gpu_seconds"],
            "unit": "GPU-s", "higher_is_better": False, "impl": "gb300",
            "config": {"workload": name, "image": f"{edge}^3, 4 phases, porosity {por:.3f}",
                       "walkers": n, "echoes": echoes, "steps_per_echo": spe, "T2b_ms": t2b,
                       "noise_sigma": 1e-3},
            "gradient_fit": {"gpu_seconds": res["gpu_seconds"], "walks": res["walks"], "evals": res["evals"],
                             "rho": res["rho"].tolist(), "hidden_rho": hidden.tolist(), "loss": res["loss"],
                             "wall_seconds": res["wall_seconds"]},
            "ga_fit": {"gpu_seconds": ga_gpu_fit, "walks": ga.evaluations, "generations": args.ga_generations,
                       "population": 64, "rho": ga.best[0].tolist(), "fitness": ga.best[1], "loss": ga_loss,
                       "wall_seconds": ga_wall},
            "noise_floor_loss": floor,
            "gpu_seconds_ratio_ga_over_gradient": ga_gpu_fit / max(res["gpu_seconds"], 1e-12)}
    eng.close()
    return line


def fit_batch(args, small=False):
    """Batched uneven workload: 64 sphere packs with edges U[64, 320] (radii 3-15, porosity U[0.15,
    0.40], seeds 100-163), walkers U[1e4, 5e5], 16 relaxivity candidates per image, 3000 echoes of 3
    steps: one persistent histogram walk (autotuned block shape) keeps every image's per-echo collision
    histograms, then each Gauss-Newton iteration evaluates every candidate and its derivative from them
    (CUDA graph). Compared with per-image plain CPMG + the restated GA (population 64), run on every
    image for `args.ga_generations_measured` generations and scaled to `args.ga_generations`: the GPU
    time of the initial population plus that many times the measured per-generation time (diversity
    resets, which add evaluations, are not counted, so the GA figure is a lower bound). A full GA run
    on the smallest image gives the GA's accuracy. Returns the result dict."""
    from concurrent.futures import ThreadPoolExecutor

    from randomwalk_nmr_gb300 import Batch, Engine
    from randomwalk_nmr_gb300.autograd import echo_times
    from randomwalk_nmr_gb300.fit import decrease_factor, fit_rho_batch
    from randomwalk_nmr_gb300.ga import GeneticAlgorithm, misfit_fitness

    n_img = 8 if small else 64
    n_use = min(args.images or n_img, n_img)
    echoes, spe, t2b = args.echoes or (300 if small else 3000), 3, 2800.0
    rng = np.random.default_rng(100)
    specs = []
    for k in range(n_img):
        edge = int(rng.integers(64, 321)) if not small else int(rng.integers(32, 81))
        nw = int(rng.integers(10_000, 500_001)) if not small else int(rng.integers(2_000, 20_001))
        specs.append(((edge,) * 3, 3.0, 15.0, float(rng.uniform(0.15, 0.40)), 1, 100 + k, nw, 1000 + k))
    t0 = time.perf_counter()
    specs = specs[:n_use]
    n_img = n_use
    with ThreadPoolExecutor(os.cpu_count() or 4) as ex:
        imgs = list(ex.map(_sphere_image, specs))
    setup_s = time.perf_counter() - t0
    b = Batch(0)
    for lab, blocks, w, por in imgs:
        b.add_image(blocks, lab.shape, *w)
    nwalk = np.array([len(im[2][0]) for im in imgs])
    # tune on a walk long enough for the collision counts (and so the table gathers) to spread as in
    # the fit; the sweep's GPU time is reported separately from the fit's
    tuned, tuned_wpt, tune_ms = b.autotune(min(echoes, 1000), spe, 16, method=args.batch_method)
    hidden = rng.uniform(2.0, 50.0, n_img)
    fh = np.ones((n_img, 16))
    fh[:, 0] = decrease_factor(hidden)
    # targets by the candidate walk, which stores no histograms: the fit's first call does (and is
    # charged for) the histogram walk
    echo, _ = b.cpmg(fh, echoes, spe, derivatives=False, method="walk")
    bulk = np.exp(-echo_times(echoes, spe, 1.0 / 15.0) / t2b)
    targets = echo[:, 0] / nwalk[:, None] * bulk + rng.normal(0.0, 1e-3, (n_img, echoes + 1))
    rho0 = rng.uniform(2.0, 50.0, (n_img, 16))
    fit = fit_rho_batch(b, targets, nwalk, echoes, spe, t2b, rho0, iters=args.fit_iters, method=args.batch_method)
    hist_walk_s = b.histogram_walk_ms * 1e-3 if args.batch_method != "walk" else 0.0
    steps_per_pass = int(nwalk.sum()) * echoes * spe
    b.close()

    # per-image plain CPMG + GA: every image's GA runs on the GPU walk of that image
    eng = Engine(0)
    g_meas = max(1, args.ga_generations_measured)
    init_s, gen_s, evals_init, evals_gen = 0.0, 0.0, 0, 0
    for k, (lab, blocks, w, por) in enumerate(imgs):
        eng.upload_labels(lab, 1)
        eng.upload_walkers(*w)
        spent = [0.0]

        def model(g, k=k):
            m = eng.cpmg(echoes, spe, decrease_factor(g[0]))["echo_sum"]
            spent[0] += eng.last_kernel_ms * 1e-3
            return m / nwalk[k] * bulk

        ga = GeneticAlgorithm(misfit_fitness(model, targets[k], 1e-3), [2.0], [50.0], population=64, seed=5 + k)
        init_s += spent[0]
        evals_init += ga.evaluations
        spent[0] = 0.0
        e0 = ga.evaluations
        ga.run(g_meas)
        gen_s += spent[0]
        evals_gen += ga.evaluations - e0
    ga_gpu = init_s + gen_s / g_meas * args.ga_generations
    # a full GA run on the smallest image: its evaluation count and accuracy
    k0 = int(np.argmin(nwalk * np.array([im[0].size for im in imgs])))
    lab, blocks, w, por = imgs[k0]
    eng.upload_labels(lab, 1)
    eng.upload_walkers(*w)
    full_s = [0.0]

    def model0(g):
        m = eng.cpmg(echoes, spe, decrease_factor(g[0]))["echo_sum"]
        full_s[0] += eng.last_kernel_ms * 1e-3
        return m / nwalk[k0] * bulk

    ga0 = GeneticAlgorithm(misfit_fitness(model0, targets[k0], 1e-3), [2.0], [50.0], population=64, seed=5)
    ga0.run(args.ga_generations)
    eng.close()
    return {"images": n_img, "walkers_total": int(nwalk.sum()), "echoes": echoes, "steps_per_echo": spe,
            "candidates": 16, "walker_steps_per_pass": steps_per_pass, "autotuned_threads": tuned,
            "autotuned_walkers_per_thread": tuned_wpt, "autotune_best_walk_ms": tune_ms, "setup_seconds": setup_s,
            "batched_fit": {"gpu_seconds": fit["gpu_seconds"], "passes": fit["walks"],
                            "method": "walk" if args.batch_method == "walk" else "histograms",
                            "histogram_walk_seconds": hist_walk_s,
                            "histogram_walk_walker_steps_per_s": steps_per_pass / hist_walk_s if hist_walk_s else None,
                            "evaluation_ms_per_pass": ((fit["gpu_seconds"] - hist_walk_s) * 1e3 / fit["walks"]
                                                       if hist_walk_s else None),
                            "candidate_walk_walker_steps_per_s": (None if hist_walk_s else
                                                                  steps_per_pass * fit["walks"] / fit["gpu_seconds"]),
                            "max_abs_rho_error": float(np.max(np.abs(fit["rho"] - hidden))),
                            "median_abs_rho_error": float(np.median(np.abs(fit["rho"] - hidden)))},
            "per_image_cpmg_ga": {"gpu_seconds": ga_gpu, "measured_gpu_seconds": init_s + gen_s,
                                  "initial_population_gpu_seconds": init_s, "initial_population_evaluations": evals_init,
                                  "measured_generations": g_meas, "measured_generation_gpu_seconds": gen_s,
                                  "measured_generation_evaluations": evals_gen, "generations": args.ga_generations,
                                  "population": 64,
                                  "method": (f"GA run on every image for {g_meas} generation(s) on that image's GPU "
                                             f"walk; GPU time = initial population + {args.ga_generations} x the "
                                             "measured per-generation time (diversity resets not counted: a lower "
                                             "bound)"),
                                  "full_run_smallest_image": {"generations": args.ga_generations,
                                                              "evaluations": ga0.evaluations,
                                                              "gpu_seconds": full_s[0],
                                                              "abs_rho_error": float(abs(ga0.best[0][0] - hidden[k0])),
                                                              "batched_fit_abs_rho_error":
                                                                  float(abs(fit["rho"][k0] - hidden[k0]))}},
            "gpu_seconds_ratio_ga_over_batched": ga_gpu / max(fit["gpu_seconds"], 1e-12)}


def run_fit_batch(args):
    r = fit_batch(args, args.workload.endswith("-small"))
    line = {"metric": "GPU-seconds of the relaxivity fit over uneven images (batched+adjoint vs per-image CPMG+GA)",
            "value": r["batched_fit"]["gpu_seconds"], "unit": "GPU-s", "higher_is_better": False, "impl": "gb300",
            "config": dict({k: v for k, v in r.items() if not isinstance(v, dict)}, workload=args.workload)}
    line.update({k: v for k, v in r.items() if isinstance(v, dict)})
    line["gpu_seconds_ratio_ga_over_batched"] = r["gpu_seconds_ratio_ga_over_batched"]
    print(json.dumps(line))


def pfgse_setup(small, direction=(0.0, 0.0, 1.0)):
    """PFGSE diffusion workload: 256^3 sphere pack (radii 5-15, porosity 0.35, seed 3), 1M walkers
    (SEED 7), rho 10 um/s, D0 2.5, 1 um voxels; 64 gradients linear 0-100 G/cm along z (or along
    `direction`), delta 1 ms, 10 exposure times log-spaced 1-100 ms (15 ... 1500 steps, walked
    cumulatively)."""
    shape = (128, 128, 128) if small else (256, 256, 256)
    walkers = 100_000 if small else 1_000_000
    w = dict(name="pfgse-256" + ("-small" if small else ""), shape=shape, rmin=5.0, rmax=15.0, porosity=0.35,
             n_phases=1, img_seed=3, walkers=walkers, seed=7, rho=[10.0], d0=2.5, bc="noflux")
    res = 1.0
    dt = res * res / (6.0 * w["d0"])
    deltas = 10.0 ** np.linspace(0.0, 2.0, 10)
    steps = np.array([max(1, int(round(d / dt))) for d in deltas], np.int32)
    n_g, gmax, pulse, gamma = 64, 100.0, 1.0, 42.576 * 2.0 * np.pi
    g = np.arange(n_g) * (gmax / (n_g - 1))
    d = np.asarray(direction, np.float64)
    kvec = np.outer((pulse * 1e-3) * (gamma * 1e6) * (g * 1e-8), d / np.linalg.norm(d))  # NMR_pfgse.cpp:483-486
    f = 1.0 - (2.0 / 3.0) * (np.asarray(w["rho"]) * res) / (w["d0"] * 1e3)
    return w, res, steps, kvec, f, deltas


def run_pfgse(args):
    direction = tuple(float(v) for v in args.gradient_direction.split(","))
    small = args.workload.endswith("-small")
    if args.impl != "reference":
        print(json.dumps(pfgse_measure(args, small, direction)))
        return
    w, res, steps, kvec, f, deltas = pfgse_setup(small, direction)
    if args.impl == "reference":
        # reference arm: the reference's CPU PFGSE walk and phase sums (oracle port) on a bounded sample
        if int(os.environ.get("RANK", "0")) != 0:
            return
        o, labels, por, walkers = oracle_inputs(w)
        threads = os.cpu_count() or 1
        m = min(len(walkers[0]), 64 * 1024)
        sample = tuple(a[:m] for a in walkers)
        for _ in range(args.warmup):
            o.pfgse(labels, sample, f, steps[:3], kvec, res, threads=threads)
        ts = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            o.pfgse(labels, sample, f, steps, kvec, res, threads=threads)
            ts.append(time.perf_counter() - t0)
        v = m * int(steps[-1]) / statistics.mean(ts)
        print(json.dumps({"impl": "reference", "metric": "walker-steps/s (PFGSE)", "value": v, "unit": "walker-steps/s",
                          "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": statistics.mean(ts) * 1e3, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "data": "synthetic sphere pack",
                          "config": {"workload": w["name"], "walkers_sampled": m},
                          "cpu_baseline": {"value": v, "unit": "walker-steps/s", "cores": threads, "kind": "port",
                                           "sample": f"first {m} walkers, all 10 exposure times"},
                          "e2e": {"value": v, "unit": "walker-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return


def pfgse_measure(args, small, direction):
    """The PFGSE workload on the GPU (see pfgse_setup); returns the result line."""
    import torch

    from randomwalk_nmr_gb300 import Engine

    w, res, steps, kvec, f, deltas = pfgse_setup(small, direction)
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    labels, por, walkers = build_inputs(w)
    n = len(walkers[0])
    steps_per_run = n * int(steps[-1])
    eng = Engine(local)
    eng.upload_labels(labels, 1)
    eng.upload_walkers(*walkers)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    for _ in range(max(3, args.warmup)):
        out = eng.pfgse(steps, kvec, res, f)
    launches0 = eng.launch_count
    kernel_s = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            out = eng.pfgse(steps, kvec, res, f)
            kernel_s.append(eng.last_kernel_ms * 1e-3)
        torch.cuda.synchronize()
    launches = eng.launch_count - launches0
    t_step = statistics.mean(kernel_s)
    value = steps_per_run / t_step
    e2e = None
    if not args.no_e2e:
        lab_p = torch.from_numpy(labels).pin_memory()
        wp = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in walkers]
        e2e_s = []
        for k in range(args.steps + 1):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            eng.upload_labels(lab_p.numpy(), 1)
            eng.upload_walkers(*[t.numpy() for t in wp])
            o2 = eng.pfgse(steps, kvec, res, f)
            t1 = time.perf_counter()
            if k:
                e2e_s.append(t1 - t0)
        assert np.array_equal(o2["M"], out["M"])
        te = statistics.mean(e2e_s)
        e2e = {"value": steps_per_run / te, "unit": "walker-steps/s",
               "h2d_bytes_per_step": int(labels.nbytes + sum(a.nbytes for a in walkers)),
               "d2h_bytes_per_step": int(out["M"].nbytes + out["esum"].nbytes + out["msd"].nbytes), "ms_per_step": te * 1e3}
    peak, peak_kind, peaks = measured_peaks()
    achieved = steps_per_run * 4 / t_step / 1e9
    clk_sum = clk.summary()
    roofline = issue_roofline(value, steps_per_run, t_step, local, clk_sum, peaks, kernel_counters(w["name"]))
    roofline["note"] = ("one launch walks every walker to the longest exposure time; its time includes the "
                        "displacement-histogram and phase kernels")
    roofline["hbm"] = {"achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                       "peak_source": peak_kind, "note": "4 B bit-block half gathered per walker-step; L2/L1-resident"}
    base, err = None, None
    if not args.no_cpu_baseline:
        from oracle.pyoracle import Oracle, build

        build(with_ref=False)
        o = Oracle()
        threads = os.cpu_count() or 1
        x, y, z, s_ = walkers
        # calibrate on a small sample, then size the timed sample to ~12 s of host work
        m0 = min(n, 1024 * threads)
        t0 = time.perf_counter()
        o.pfgse(labels, (x[:m0], y[:m0], z[:m0], s_[:m0]), f, steps, kvec, res, threads=threads)
        rate = m0 / (time.perf_counter() - t0)
        m = int(max(m0, min(n, rate * 12.0)))
        sample = (x[:m], y[:m], z[:m], s_[:m])
        t0 = time.perf_counter()
        ob = o.pfgse(labels, sample, f, steps, kvec, res, threads=threads)
        dt_cpu = time.perf_counter() - t0
        base = dict(value=m * int(steps[-1]) / dt_cpu, unit="walker-steps/s", cores=threads, kind="port",
                    sample=f"first {m} of {n} walkers, all 10 exposure times ({dt_cpu:.1f} s)")
        sub = Engine(local)
        sub.upload_labels(labels, 1)
        sub.upload_walkers(*sample)
        og = sub.pfgse(steps, kvec, res, f)
        sub.close()
        err = float(np.max(np.abs(og["M"] - ob["M"]) / ob["M"][:, :1]))
    line = {"metric": "walker-steps/s (PFGSE)", "value": value, "unit": "walker-steps/s", "n_gpus": 1,
            "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": t_step * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32/u64 walk, exact fixed-point energy histograms, f64 phase sums",
            "data": "synthetic sphere pack (no reference benchmark data)",
            "config": {"workload": w["name"], "image": "x".join(map(str, w["shape"])), "porosity": round(por, 4),
                       "walkers": n, "gradients": int(len(kvec)), "gradient_direction": list(direction),
                       "exposure_times_ms": [round(float(d), 4) for d in deltas],
                       "steps": [int(v) for v in steps], "walker_steps_per_step": steps_per_run,
                       "l2": "flushed (512 MB write) before every timed step", "parallelism": "1 GPU"},
            "roofline": roofline,
            "cpu_baseline": base, "e2e": e2e, "gpu_launches": launches,
            "attenuation_max_err_vs_oracle": err, "clocks": clk_sum,
            "check": {"M0_equals_energy_sum": bool(np.allclose(out["M"][:, 0], out["esum"], rtol=1e-12))}}
    eng.close()
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="cpmg-2phase-400")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--ga-generations", type=int, default=50)
    ap.add_argument("--fit-evals", type=int, default=40)
    ap.add_argument("--fit-iters", type=int, default=6)
    ap.add_argument("--ga-generations-measured", type=int, default=1,
                    help="rho-fit-batch: GA generations actually run on every image (scaled to --ga-generations)")
    ap.add_argument("--no-fit", action="store_true",
                    help="default workload: skip the other configurations carried in the bench line (fits, PFGSE)")
    ap.add_argument("--echoes", type=int, default=0, help="rho-fit-batch: echo count override (profiling)")
    ap.add_argument("--gradient-direction", default="0,0,1",
                    help="pfgse workloads: gradient direction x,y,z (an oblique one takes the general phase path)")
    ap.add_argument("--images", type=int, default=0, help="rho-fit-batch: use the first N images (profiling)")
    ap.add_argument("--batch-method", default="auto", choices=["auto", "histograms", "walk"],
                    help="rho-fit-batch: histogram evaluation (auto) or a candidate walk per fit iteration")
    args = ap.parse_args()
    if args.workload.startswith("rho-fit-multiphase"):
        return run_fit_multiphase(args)
    if args.workload.startswith("rho-fit-batch"):
        return run_fit_batch(args)
    if args.workload.startswith("pfgse-256"):
        return run_pfgse(args)
    w = workload(args.workload)
    if args.impl == "reference":
        return run_reference(args, w)

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from randomwalk_nmr_gb300 import Engine, fx_to_float

    res, spe, f = derived(w)
    # N > 1: weak scaling over a sharded population -- every rank walks its own 1M walkers (placed
    # with SEED + rank) and the per-echo limb sums are added across ranks with one exact integer
    # all-reduce (randomwalk_nmr_gb300.shard), as one GPU walking all N x 1M walkers would give
    labels, por, walkers = build_inputs(dict(w, seed=w["seed"] + rank))
    n = len(walkers[0])
    steps_per_run = n * w["echoes"] * (2 * (spe // 2) if w.get("field") else spe)  # the field walk: 2 inversions
    eng = Engine(local)
    eng.upload_labels(labels, w["n_phases"])
    eng.upload_walkers(*walkers)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    field = w.get("field")
    gamma = 1.0e6 * 42.576 * 2.0 * np.pi
    dt_s = 1.0e-3 * res * res / (6.0 * w["d0"])

    mapping = bool(w.get("map"))

    def walk():
        if mapping:
            coll = eng.map(w["echoes"] * spe, bc=w["bc"])
            return dict(echo_sum=None, echo_fx=coll)
        if field:
            o = eng.cpmg_field(w["echoes"], spe, f, gamma, dt_s, bc=w["bc"])
            return dict(echo_sum=o["echo_sum"], echo_fx=o["echo_sum"], phase=o["phase"])
        return eng.cpmg(w["echoes"], spe, f, bc=w["bc"])

    if field:
        eng.set_field_uniform(field[0], field[1], res)
    for _ in range(max(3, args.warmup)):
        walk()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches0 = eng.launch_count
    kernel_s = []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            out = walk()
            kernel_s.append(eng.last_kernel_ms * 1e-3)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    if dist and not field and not mapping:
        from randomwalk_nmr_gb300.shard import combine_cpmg

        out = combine_cpmg(out)  # the whole population's echo train on every rank
    launches = eng.launch_count - launches0
    t_step = statistics.mean(kernel_s)
    if dist:
        tt = torch.tensor([t_step], device=f"cuda:{local}")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_step = float(tt.item())
    value = world * steps_per_run / t_step

    # end to end through the C ABI from pinned host memory
    e2e = None
    if not args.no_e2e:
        lab_p = torch.from_numpy(labels).pin_memory()
        wp = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in walkers]
        e2e_s = []
        for k in range(args.steps + 1):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            eng.upload_labels(lab_p.numpy(), w["n_phases"])
            eng.upload_walkers(*[t.numpy() for t in wp])
            if field:
                eng.set_field_uniform(field[0], field[1], res)
            o2 = walk()
            if dist and not field and not mapping:
                o2 = combine_cpmg(o2)
            t1 = time.perf_counter()
            if k:
                e2e_s.append(t1 - t0)
        assert np.array_equal(o2["echo_fx"], out["echo_fx"])
        h2d = labels.nbytes + sum(a.nbytes for a in walkers)
        d2h = (w["echoes"] + 1) * (3 + (1 if w["n_phases"] == 1 else (2 if w["n_phases"] == 2 else 4))) * 8 + 4
        if field:
            d2h = (w["echoes"] + 1) * 3 * 8 + 4 + n * 8  # echo limbs, status, final phases
        if mapping:
            d2h = n * 4 + 4  # per-walker collision counts, status
        te = statistics.mean(e2e_s)
        if dist:
            tt = torch.tensor([te], device=f"cuda:{local}")
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            te = float(tt.item())
        e2e = {"value": world * steps_per_run / te, "unit": "walker-steps/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": te * 1e3}

    peak, peak_kind, peaks = measured_peaks()
    words = 1 if w["n_phases"] == 1 else (2 if w["n_phases"] == 2 else 4)
    gather_bytes = 4 * words  # algorithmic bytes gathered per walker-step: one 32-bit half of each block word
    launches_per_walk = max(1, launches // max(1, args.steps))
    counters = kernel_counters(w["name"])
    clk_sum = clk.summary()
    roofline = issue_roofline(value / world, steps_per_run / launches_per_walk, t_step / launches_per_walk, local,
                              clk_sum, peaks, counters)
    roofline["hbm"] = {"achieved": steps_per_run * gather_bytes / t_step / 1e9, "peak": peak, "unit": "GB/s",
                       "frac": steps_per_run * gather_bytes / t_step / 1e9 / peak, "peak_source": peak_kind,
                       "traffic": counters.get("dram_bytes_per_launch"), "traffic_unit": "bytes per launch",
                       "note": "bit-block bytes gathered per walker-step (4 B per block word) x walker-steps / walk-"
                               "kernel time, against the measured HBM copy peak; the gathers are served on chip "
                               "(L1 hits), so this roof does not bind"}
    roofline["launches_per_walk"] = launches_per_walk
    if field:
        # the reference's phase updates: two FP64 fused multiply-adds per step, kept bit for bit
        roofline["fp64"] = {"dfma_per_walker_step": 2, "achieved_tflops": (value / world) * 2 * 2 / 1e12,
                            "pipe_active_pct_ncu": counters.get("fp64_pipe_pct"),
                            "note": "no measured FP64 peak on this pool; ncu's FP64 pipe utilisation is the fraction"}

    base = None
    echo_err = None
    if rank == 0 and not args.no_cpu_baseline and field:
        # the oracle's field walk on a bounded sample; phases bit-exact, echo sums to 1e-12 * n
        from oracle.pyoracle import Oracle, build

        build(with_ref=False)
        o = Oracle()
        threads = os.cpu_count() or 1
        m = min(n, 256 * threads)
        sample = tuple(a[:m] for a in walkers)
        gt = 0.5 * gamma * dt_s
        dg = field[0] * 1.0e-6 * res
        t0 = time.perf_counter()
        ob = o.cpmg_field(labels, sample, w["echoes"], spe, f, gt, dg=dg, axis=field[1], bc=w["bc"],
                          n_phases=w["n_phases"], threads=threads)
        dt_cpu = time.perf_counter() - t0
        base = dict(value=m * w["echoes"] * 2 * (spe // 2) / dt_cpu, unit="walker-steps/s", cores=threads, kind="port",
                    sample=f"first {m} of {n} walkers, all {w['echoes']} echoes ({dt_cpu:.1f} s)")
        sub = Engine(local)
        sub.upload_labels(labels, w["n_phases"])
        sub.upload_walkers(*sample)
        sub.set_field_uniform(field[0], field[1], res)
        og = sub.cpmg_field(w["echoes"], spe, f, gamma, dt_s, bc=w["bc"])
        sub.close()
        echo_err = float(np.max(np.abs(og["echo_sum"] - ob["echo_fp64"])) / m)
        assert np.array_equal(og["phase"].view(np.uint64), ob["phasef"].view(np.uint64)), "phases differ from the oracle"
    elif rank == 0 and not args.no_cpu_baseline and mapping:
        # the CPU walk of the oracle (the mapping walk's steps plus the energy update) on a sample;
        # the GPU mapping walk's per-walker collision counts on that sample must equal the oracle's
        base, ob, sample = cpu_baseline(labels, w["n_phases"], walkers, spe, w["echoes"], f, w["bc"])
        sub = Engine(local)
        sub.upload_labels(labels, w["n_phases"])
        sub.upload_walkers(*sample)
        cm = sub.map(w["echoes"] * spe, bc=w["bc"])
        sub.close()
        assert np.array_equal(cm, np.asarray(ob["collf"]).reshape(len(cm), -1).sum(axis=1)), \
            "collision counts differ from the oracle"
        echo_err = 0.0
    elif rank == 0 and not args.no_cpu_baseline:
        base, ob, sample = cpu_baseline(labels, w["n_phases"], walkers, spe, w["echoes"], f, w["bc"])
        # echo error of the GPU walk against the FP64 oracle on the same walker sample
        sub = Engine(local)
        sub.upload_labels(labels, w["n_phases"])
        sub.upload_walkers(*sample)
        og = sub.cpmg(w["echoes"], spe, f, bc=w["bc"])
        sub.close()
        echo_err = float(np.max(np.abs(og["echo_sum"] - ob["echo_fp64"]) / ob["echo_fp64"]))
        assert np.array_equal(og["echo_coll"], ob["echo_coll"]), "per-echo collision counts differ from the oracle"

    if rank == 0:
        line = {"metric": ("walker-steps/s (collision-mapping walk)" if mapping else
                           "walker-steps/s (CPMG in an internal field)" if field else "walker-steps/s (plain CPMG)"),
                "value": value, "unit": "walker-steps/s", "n_gpus": world,
                "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": t_step * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": ("int32/u64 walk, u32 collision counts" if mapping else
                          "int32/u64 walk, exact 64-bit fixed-point echo sums, f64 output"),
                "data": "synthetic sphere pack (no reference benchmark data)",
                "config": {"workload": w["name"], "image": "x".join(map(str, w["shape"])), "porosity": round(por, 4),
                           "phases": w["n_phases"], "walkers": n, "echoes": w["echoes"], "steps_per_echo": spe,
                           "walker_steps_per_step": steps_per_run, "voxel_um": res, "bc": w["bc"],
                           "l2": "flushed (512 MB write) before every timed step",
                           "parallelism": (f"walkers sharded over {world} GPUs ({n} per GPU), exact integer "
                                           "all-reduce of the echo limb sums") if world > 1 else "1 GPU"},
                "roofline": roofline, "cpu_baseline": base, "e2e": e2e, "gpu_launches": int(launches),
                ("collision_counts_max_abs_diff_vs_oracle" if mapping else
                 "echo_max_abs_err_per_walker_vs_oracle" if field else "echo_max_rel_err_vs_fp64_oracle"): echo_err,
                "clocks": clk_sum}
        if not mapping:
            line["echo_check"] = float(out["echo_sum"][-1] / out["echo_sum"][0])
    eng.close()
    if rank == 0:
        if w["name"] == "cpmg-2phase-400" and world == 1 and not args.no_fit:
            # the second headline figure: GPU-seconds of the batched relaxivity fit over 64 uneven
            # images against per-image plain CPMG + GA on the same GPU (the rho-fit-batch workload)
            line["rho_fit_batch"] = fit_batch(args)
            # the other benchmark configurations measured in the same run: the PFGSE diffusion walk
            # (256^3, 64 gradients x 10 exposure times) and the differentiable multi-phase fit
            line["pfgse_256"] = pfgse_measure(args, False, (0.0, 0.0, 1.0))
            line["rho_fit_multiphase"] = fit_multiphase(args, False, "rho-fit-multiphase")
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
