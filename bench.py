"""Benchmark: nadir upwelling radiance of the 60-layer, 500,000-line,
500-2500 cm-1 column (seven absorbers, synthetic continuum), i.e. per-layer
line-by-line optical depth + far wings + continuum + the layer radiance merge.

Metric: layer-spectral-points/s = sum over layers of the layer-grid points
(what ODLAY returns per layer) / time of one full column.

  value            mixed path (FP32 line shape, Kahan sums, FP64 index math),
                   line list already resident on the device, radiance left on
                   the device; timed with CUDA events on the library's stream
  e2e              the same call through the C-ABI with host buffers: the line
                   list is copied in from pinned host memory and the radiance
                   copied back to pinned host memory inside every step
  plain            the FP64 GPU path on the same column (reported beside)
  cpu_baseline     the FP64 CPU restatement of the reference on the whole
                   column, all host threads (and one thread on six layers);
                   every GPU radiance of the run is compared with its radiance
                   (max_rel_err_vs_oracle)
  --impl reference the reference's CPU path (the FP64 restatement, all host
                   threads) on the whole column every step

Inputs are larger than L2 (the line list alone is 20 MB, the per-layer
working set of a few layers exceeds 129 MB), so no extra L2 flush is done.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "layer-spectral-points/s"
UNIT = "layer-points/s"
WORKLOAD = "60-layer nadir radiance, 500000 lines (7 absorbers), 500-2500 cm-1, synthetic continuum"


def max_over_ranks(ms, device):
    """Slowest rank's time: every rank runs a full replica of the workload."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(points_per_replica, world, ms):
    """Whole-job throughput of `world` replicas finishing within `ms`."""
    return points_per_replica * world / (ms * 1e-3)


FLOP_CNVFNQ = 19   # per CNVFNQ inner step (R3, R2, R1 updates of one line at one point)
FLOP_CNVF4Q = 9    # per CNVF4Q inner step (one far-wing record at one R4 point)


def fp32_peak_tflops():
    """Nominal FP32 FMA rate (152 SMs x 128 lanes x 2 FLOP) at the measured
    maximum SM clock of the GB300s."""
    mhz = 2070.0
    try:
        mhz = float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["sm_max_mhz"])
    except Exception:
        pass
    return 152 * 128 * 2 * mhz * 1e6 / 1e12, mhz


def hbm_peak_gbs():
    """Measured copy bandwidth of the GB300s (GB/s), else the 6.8 TB/s fallback."""
    try:
        return float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
    except Exception:
        return 6800.0


def load_traffic():
    """DRAM bytes per output point of each kernel, from the ncu capture whose
    summary profiles/dram_traffic.txt holds (lines `kernel bytes_per_point`;
    a kernel without a line reports traffic null)."""
    out = {}
    try:
        for line in (ROOT / "profiles" / "dram_traffic.txt").read_text().splitlines():
            f = line.split()
            if len(f) == 2 and not line.startswith("#"):
                out[f[0]] = float(f[1])
    except (OSError, ValueError):
        pass
    return out


def roofline(work, kt, steps, ms_step, points):
    """Roofline of the dominant line-shape kernel: algorithmic FLOPs of one
    launch (the call's step counts) over its CUDA-event time on the library's
    stream, averaged over the timed steps; `points` (the launch's output
    points) scales the measured DRAM bytes per point to the launch."""
    peak, mhz = fp32_peak_tflops()
    traffic = load_traffic()
    kernels = {
        "k_f4_conv": (FLOP_CNVF4Q * work["cnvf4q_steps"], kt["ms_f4conv"] / steps, work["cnvf4q_steps"]),
        "k_panel": (FLOP_CNVFNQ * work["cnvfnq_steps"], kt["ms_panel"] / steps, work["cnvfnq_steps"]),
    }
    out = {}
    for name, (flop, ms, nstep) in kernels.items():
        ach = flop / (ms * 1e-3) / 1e12 if ms > 0 else None
        bpp = traffic.get(name)
        out[name] = {"bound": "fp32", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                     "frac": ach / peak if ach else None,
                     "traffic": bpp * points if bpp is not None else None,
                     "traffic_source": ("scaled from a stored ncu capture: DRAM bytes per output point "
                                        "(profiles/dram_traffic.txt) x this launch's points"
                                        if bpp is not None else None),
                     "ms_per_launch": ms, "share_of_step": ms / ms_step, "flop_per_launch": flop}
    if kt.get("ms_rt", 0) > 0 and work.get("rt_bytes", 0) > 0:
        # the layer recurrence (one launch per run of layers on one merge
        # grid): algorithmic bytes over its device time, against the measured
        # copy bandwidth
        hbm = hbm_peak_gbs()
        ms_rt = kt["ms_rt"] / steps
        ach = work["rt_bytes"] / (ms_rt * 1e-3) / 1e9
        bpp = traffic.get("k_rt_segment")
        out["k_rt_segment"] = {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                               "traffic": bpp * points if bpp is not None else None,
                               "traffic_source": ("scaled from a stored ncu capture: DRAM bytes per layer point "
                                                  "(profiles/dram_traffic.txt) x this step's layer points"
                                                  if bpp is not None else None),
                               "ms_per_step": ms_rt, "share_of_step": ms_rt / ms_step,
                               "bytes_per_step": work["rt_bytes"],
                               "bytes_counted": "every layer's OD once, the merged radiance and reflectance in and "
                                                "out once per run of layers on one merge grid",
                               "peak_source": "hbm_gbs of MEASURED_PEAKS.json (burst copy)"}
    top = max((k for k in out if out[k]["bound"] == "fp32"), key=lambda k: out[k]["ms_per_launch"])
    r = dict(out[top])
    r["kernel"] = top
    r["peak_source"] = ("nominal FP32 FMA rate, 152 SMs x 128 lanes x 2 FLOP x %.0f MHz (sm_max_mhz of "
                        "MEASURED_PEAKS.json, which holds no FP32 figure)" % mhz)
    r["others"] = {k: v for k, v in out.items() if k != top}
    return r


def od_points(v1, v2, dv_normal, dv_narrow):
    """Points ODLAY returns for one layer on its own grid: the grid choice of
    clblm_ODLAY.f90:443-457 (DVnarrow when within 20 %) and panelOut's panel
    rule (:2349-2360): panels of 2400 points from VFT = V1 - 32 DV until the
    panel reaching V2, whose NHI is cut there (one more point when the cut
    falls short of V2).  The same arithmetic as clblm_gpu_od_size; binary64
    throughout, with no fused operations."""
    dv = dv_normal if abs(dv_normal - dv_narrow) / dv_normal > 0.2 else dv_narrow
    vft = v1 - 32.0 * dv
    nhi0 = 2401 + 32 - 1
    n = 0
    while True:
        if vft + (nhi0 - 1) * dv > v2:
            nhi = int((v2 - vft) / dv + 1.0)
            if vft + (nhi - 1) * dv < v2:
                nhi += 1
            return n + nhi - 33 + 1
        n += nhi0 - 33 + 1
        vft = vft + 2400.0 * dv


def layer_points_host(col, ctrl):
    """Sum over layers of the points ODLAY returns on each layer grid, from
    setDV (the oracle's, no device) and the panel rule (od_points)."""
    from oracle import oracle as O
    dn, df, _ = O.Session().setdv(col, ctrl.sample, ctrl.alfal0, ctrl.alfal0_fine, ctrl.grid_type, ctrl.dv_user)
    return sum(od_points(col.v1, col.v2, dn[il], df[il]) for il in range(col.nlay))


def layer_points(h, col, ctrl):
    """Sum over layers of the points ODLAY returns on each layer grid."""
    from clblm_gb300 import capi
    from clblm_gb300 import capi_types as T
    dn, df, do = capi.setDV(col, ctrl.sample, ctrl.alfal0, ctrl.alfal0_fine, ctrl.grid_type, ctrl.dv_user)
    tot = 0
    for il in range(col.nlay):
        g = T.grid_struct(col.v1, col.v2, dn[il], df[il], do, ctrl.sample, ctrl.alfal0)
        n, _ = h.od_size(col.layer(il), g, ctrl.od)
        tot += n
    return tot


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                                      "--query-gpu=" + self.Q, "--format=csv,noheader,nounits"],
                                     capture_output=True, text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.splitlines()[0].split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k].strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def pinned_lines(lines):
    """Copy of a line list whose arrays live in pinned host memory."""
    import torch
    from clblm_gb300.capi_types import Lines
    arrs = {}
    keep = []
    for name, dt in Lines.FIELDS:
        src = getattr(lines, name)
        t = torch.empty(src.nbytes, dtype=torch.uint8, pin_memory=True)
        a = t.numpy().view(dt)
        a[:] = src
        arrs[name] = a
        keep.append(t)
    pl = Lines(**arrs)
    pl._pinned = keep
    return pl


CPU_LAYERS = list(range(28, 34))     # single-thread sample: 6 adjacent layers


def cpu_sample_column(col, layers=CPU_LAYERS):
    """Adjacent layers of the column (the reference STOPs on DV ratios > 2.5
    between neighbouring layers, so the sample keeps them adjacent)."""
    return col.sub(layers)


def run_cpu(lines, col, cont, ctrl, threads, layers=None):
    """The FP64 restatement of the reference's path on `threads` host threads
    (layer ODs in parallel, the merge's per-point loops in parallel): the
    radiance of `col` (or of its `layers`), its sub-column and the time."""
    from oracle import oracle as O
    s = O.Session()
    sub = col if layers is None else cpu_sample_column(col, layers)
    t0 = time.perf_counter()
    rad, _ = s.rt_mode2(lines, sub, ctrl, cont, nthreads=threads)
    dt = time.perf_counter() - t0
    return sub, dt, rad


def rel_err(got, ref):
    """Largest relative difference |got - ref| / |ref| over the spectrum."""
    got, ref = np.asarray(got, dtype=np.float64), np.asarray(ref, dtype=np.float64)
    if got.shape != ref.shape:
        return None
    return float(np.max(np.abs(got - ref) / np.abs(ref)))


def jacobian_leg(cont, steps):
    """Radiance plus the level-temperature and ln q(H2O) Jacobians of every
    level of the 60-layer column over 600-1100 cm-1 (the 120,000 lines of the
    500,000-line list there), on the uniform grid of noScattJacob: mixed path
    timed, FP64 path timed once, and their radiance and Jacobian agreement."""
    import torch
    from clblm_gb300 import capi, synth
    from clblm_gb300 import capi_types as T
    lines, col, _ = synth.config1()
    lines, col = lines.window(600.0, 1100.0), col.with_window(600.0, 1100.0)
    prof = synth.jac_profile(col)
    h = capi.Handle(lines, cont)
    res = {}
    outs = {}
    for name, prec, k in (("mixed", T.CLBLM_PREC_MIXED, steps), ("plain", T.CLBLM_PREC_PLAIN, 1)):
        ctrl = T.rt_ctrl(precision=prec, grid_type=1)
        n, dv = h.jac_size(col, ctrl, prof)
        nl = col.nlay
        o = {key: torch.empty(shape, dtype=torch.float64, device="cuda")
             for key, shape in (("rad", n), ("dtlev", (nl + 1, n)), ("dqlev", (nl + 1, n)), ("dtsfc", n),
                                ("demis", n))}
        call = lambda: h.jac_device(col, ctrl, prof, o["rad"].data_ptr(), o["dtlev"].data_ptr(),
                                    o["dqlev"].data_ptr(), o["dtsfc"].data_ptr(), o["demis"].data_ptr(), n)
        call()  # warm-up (workspace growth)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(k):
            call()
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1e3 / k
        res[name] = {"ms_per_step": ms, "value": n * nl / (ms * 1e-3)}
        outs[name] = {key: v.clone() for key, v in o.items()}
        res["points"], res["dv"], res["layers"] = n, dv, nl
    m, p = outs["mixed"], outs["plain"]
    res["max_rel_rad_diff_mixed_vs_plain"] = float(((m["rad"] - p["rad"]).abs() / p["rad"].abs()).max())
    for key in ("dtlev", "dqlev"):
        # max |mixed - FP64| over the largest |FP64| Jacobian of all levels
        # (levels under an opaque lower atmosphere have Jacobians near 1e-50,
        # below FP32's range, so a per-level ratio says nothing); levels that
        # are not finite in FP64, if any, are left out
        ok = torch.isfinite(p[key]).all(dim=1)
        scale = p[key][ok].abs().max()
        d = (m[key][ok] - p[key][ok]).abs().max()
        res["max_%s_diff_mixed_vs_plain" % key] = float(d / scale) if ok.any() and scale > 0 else None
        res["levels_compared_%s" % key] = int(ok.sum())
    res["unit"] = UNIT
    res["workload"] = ("60-layer column, 120k lines, 600-1100 cm-1: radiance + dR/dT and dR/dln q(H2O) of all "
                       "61 levels (noScattJacob, 100000-point blocks, uniform DV)")
    res["speedup_mixed_vs_plain"] = res["plain"]["ms_per_step"] / res["mixed"]["ms_per_step"]
    h.close()
    return res


def autograd_leg(cont, steps):
    """The radiance of the 60-layer column over 600-1100 cm-1 as a
    differentiable function of its level profile (torch.autograd): forward
    (layers from the levels by ALAYER + FPACK, then the radiance alone) and
    backward (the vector-Jacobian product of clblm_gpu_jac_vjp: the layer ODs
    formed again block by block and every block's derivatives reduced against
    the gradient), mixed path; the backward's agreement with the dense
    Jacobians contracted with the same gradient (one FP64 call each)."""
    import torch
    from clblm_gb300 import capi, synth, torch_ops
    from clblm_gb300 import capi_types as T
    lines, col, _ = synth.config1()
    lines, col = lines.window(600.0, 1100.0), col.with_window(600.0, 1100.0)
    h = capi.Handle(lines, cont)
    ctrl = T.rt_ctrl(precision=T.CLBLM_PREC_MIXED, grid_type=1)
    p = torch_ops.RadianceProblem.from_column(h, ctrl, col)
    t0, q0 = p.levels(np.append(col.tbot, col.ttop[-1]))
    ts = torch.tensor(col.tskin, dtype=torch.float64, device="cuda")
    em = torch.tensor(col.emis, dtype=torch.float64, device="cuda")

    def step():
        t = t0.clone().requires_grad_()
        q = q0.clone().requires_grad_()
        torch.cuda.synchronize()
        a = time.perf_counter()
        rad = torch_ops.nadir_radiance(p, t, q, ts, em)
        torch.cuda.synchronize()
        b = time.perf_counter()
        rad.sum().backward()
        torch.cuda.synchronize()
        c = time.perf_counter()
        return (b - a) * 1e3, (c - b) * 1e3, len(rad), t.grad

    step()  # warm-up
    fw, bw = [], []
    for _ in range(steps):
        f_ms, b_ms, n, gt = step()
        fw.append(f_ms)
        bw.append(b_ms)
    res = {"workload": "60-layer column, 120k lines, 600-1100 cm-1: radiance of the level profile (forward) and "
                       "the gradient of its sum with respect to the 61 level temperatures and ln q(H2O), Tskin "
                       "and emissivity (backward: vector-Jacobian product, no stored Jacobian)",
           "points": n, "forward_ms": float(np.min(fw)), "backward_ms": float(np.min(bw)),
           "forward_plus_backward_ms": float(np.min(fw) + np.min(bw)), "steps": steps}
    # against the dense Jacobians (FP64 both)
    c0, prof0 = p.state(np.append(col.tbot, col.ttop[-1]), q0.cpu().numpy(), col.tskin, col.emis)
    pc = T.clblm_rt_ctrl_t.from_buffer_copy(p.ctrl)
    pc.od.precision = T.CLBLM_PREC_PLAIN
    g = np.random.default_rng(0).standard_normal(n)
    dense = h.jac(c0, pc, prof0)
    v = h.jac_vjp(c0, pc, prof0, g)
    want = dense["dtlev"] @ g
    # relative to the largest level gradient: a level the radiance does not
    # depend on has a zero gradient in both
    res["fp64_vjp_vs_dense_jacobians_max_rel"] = float(np.max(np.abs(v["g_tlev"] - want)) / np.max(np.abs(want)))
    h.close()
    return res


def batch_leg(cont, steps, per_call=16):
    """Batched profiles: 256 seeded profiles (20-100 layers, level
    temperatures + N(0, 3 K), windows of log-uniform width 10-1000 cm-1 in
    500-2500 cm-1), each with radiance and T / ln q(H2O) Jacobians of every
    level, through clblm_gpu_batch in calls of `per_call` profiles whose
    launch sequences are captured once as CUDA graphs and replayed (outputs
    in a device pool reused by the calls).  The mixed path is timed; the
    first call's profiles are also run in FP64 for the agreement."""
    import torch
    from clblm_gb300 import capi, synth
    from clblm_gb300 import capi_types as T
    lines, _, cols, jacs = synth.config3()
    h = capi.Handle(lines, cont)
    ctrl = T.rt_ctrl(precision=T.CLBLM_PREC_MIXED, grid_type=1)
    groups = [list(range(i, min(i + per_call, len(cols)))) for i in range(0, len(cols), per_call)]
    sizes = []
    for g in groups:
        n, _ = h.batch_size([cols[i] for i in g], ctrl, [jacs[i] for i in g])
        sizes.append(n)
    # one device pool, laid out per call
    need = max(sum(n * (3 + 2 * (cols[i].nlay + 1)) for n, i in zip(ns, g)) for ns, g in zip(sizes, groups))
    pool = torch.empty(need, dtype=torch.float64, device="cuda")
    base = pool.data_ptr()
    outs = []
    for ns, g in zip(sizes, groups):
        o, off = [], 0
        for n, i in zip(ns, g):
            nl = cols[i].nlay
            ptr = lambda k: base + 8 * (off + k)
            o.append({"rad": ptr(0), "dtsfc": ptr(n), "demis": ptr(2 * n), "dtlev": ptr(3 * n),
                      "dqlev": ptr(3 * n + (nl + 1) * n), "cap": n})
            off += n * (3 + 2 * (nl + 1))
        outs.append(o)

    def step(graph=True, prec_ctrl=ctrl, which=None):
        for k, g in enumerate(groups):
            if which is not None and k != which:
                continue
            st = h.batch_device([cols[i] for i in g], prec_ctrl, [jacs[i] for i in g], outs[k], graph=graph)
            assert not any(st), st

    step()  # first call of each group: plans, capture, run
    step()  # the sticky JRAD has settled: this is the batch that the timed steps replay
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3 / steps
    lp = sum(n * cols[i].nlay for ns, g in zip(sizes, groups) for n, i in zip(ns, g))
    res = {"workload": "256 profiles, 20-100 layers, windows 10-1000 cm-1 in 500-2500, radiance + dR/dT and "
                       "dR/dln q(H2O) of every level (clblm_gpu_batch, %d profiles per call, CUDA graphs)" % per_call,
           "profiles": len(cols), "points": int(sum(sum(ns) for ns in sizes)), "layer_points_per_step": int(lp),
           "ms_per_step": ms, "value": lp / (ms * 1e-3), "unit": UNIT, "steps": steps,
           # each layer's OD is formed four times on the Jacobian grid: the
           # viewing path, T + 1 K, Wtot * 1.01 and the H2O-only layer
           # (drv_LevelTemp, drv_LevelConc), besides the Jacobian recurrence
           "od_layer_points_per_step": int(4 * lp), "od_value": 4 * lp / (ms * 1e-3),
           "od_note": "layer OD points formed per second: 4 ODs per layer (viewing, T+1 K, Wtot*1.01, H2O alone)"}
    # agreement with FP64 on the first call's profiles (the calls share the
    # pool: the first call runs again before its radiances are kept)
    step(which=0)
    torch.cuda.synchronize()
    rad_m = [pool[o["rad"] // 8 - base // 8:o["rad"] // 8 - base // 8 + o["cap"]].clone() for o in outs[0]]
    t1 = time.perf_counter()
    step(graph=False, prec_ctrl=T.rt_ctrl(precision=T.CLBLM_PREC_PLAIN, grid_type=1), which=0)
    torch.cuda.synchronize()
    res["plain_first_call_ms"] = (time.perf_counter() - t1) * 1e3
    diff = 0.0
    for o, m in zip(outs[0], rad_m):
        p = pool[o["rad"] // 8 - base // 8:o["rad"] // 8 - base // 8 + o["cap"]]
        diff = max(diff, float(((m - p).abs() / p.abs()).max()))
    res["max_rel_rad_diff_mixed_vs_plain_first_call"] = diff
    h.close()
    del pool
    torch.cuda.empty_cache()
    return res


def config4_leg(steps, fp64_jacobians=False):
    """Broadband case: 3,000,000 lines on 10-3500 cm-1, 100 layers 1013 to
    0.01 hPa, synthetic continuum.  The nadir radiance (mixed timed, FP64
    once), its FFT scans to instrument resolution (sinc of maximum OPD
    0.8 cm, and the Gaussian of the same half width), and radiance plus the
    T and ln q(H2O) Jacobians of all 101 levels (noScattJacob, mixed)."""
    import torch
    from clblm_gb300 import capi, synth
    from clblm_gb300 import capi_types as T
    lines, col, cont = synth.config4()
    h = capi.Handle(lines, cont)
    res = {"workload": "3,000,000 lines, 10-3500 cm-1, 100 layers 1013-0.01 hPa: nadir radiance, FFT scans "
                       "(sinc OPD 0.8 cm; Gaussian), radiance + dR/dT and dR/dln q(H2O) of every level"}
    rad = {}
    for name, prec, k in (("mixed", T.CLBLM_PREC_MIXED, steps), ("plain", T.CLBLM_PREC_PLAIN, 1)):
        ctrl = T.rt_ctrl(precision=prec)
        n, dv = h.rt_size(col, ctrl)
        out = torch.empty(n, dtype=torch.float64, device="cuda")
        h.rt_mode2_device(col, ctrl, out.data_ptr(), n)  # warm-up (workspace, tuning)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(k):
            h.rt_mode2_device(col, ctrl, out.data_ptr(), n)
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1e3 / k
        st = h.stats()  # the last call's per-stream stage times (all OD batches)
        lp = layer_points(h, col, ctrl)
        res["radiance_" + name] = {"ms": ms, "value": lp / (ms * 1e-3), "unit": UNIT, "layer_points": lp,
                                   "stages_ms": {"line_chain": st["ms_line_chain"],
                                                 "far_wing_chain": st["ms_f4_chain"],
                                                 "k_f4_conv": st["ms_f4conv"], "k_panel": st["ms_panel"]}}
        res["radiance_points"], res["dv"] = n, dv
        rad[name] = out
    m, p = rad["mixed"], rad["plain"]
    res["max_rel_rad_diff_mixed_vs_plain"] = float(((m - p).abs() / p.abs()).max())
    res["radiance_speedup_mixed_vs_plain"] = res["radiance_plain"]["ms"] / res["radiance_mixed"]["ms"]
    # instrument-function scans of the mixed radiance, on the device
    hw = 1.0 / (0.8 * 3.314800)
    for name, fid in (("sinc", 5), ("gaussian", 3)):
        sc = T.scan_struct(fid, hw, 20.0, 3490.0)
        v1s, dvs, ns = capi.fftscn_size(sc, col.v1, res["dv"], len(m))
        o = torch.empty(ns, dtype=torch.float64, device="cuda")
        h.fftscn_device(sc, m.data_ptr(), len(m), col.v1, res["dv"], o.data_ptr(), ns)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(3):
            h.fftscn_device(sc, m.data_ptr(), len(m), col.v1, res["dv"], o.data_ptr(), ns)
        torch.cuda.synchronize()
        res["scan_" + name] = {"ms": (time.perf_counter() - t0) * 1e3 / 3, "hwhm": hw, "points": ns, "dv": dvs}
    del rad
    # radiance + Jacobians through the batched path (clblm_gpu_batch, one
    # profile, launched directly: the host planning is inside the timed call);
    # mixed after one warm-up call, then the same batch as a replayed CUDA
    # graph; FP64 once when asked (about 20 s)
    prof = synth.jac_profile(col)
    nl = col.nlay
    jrad = {}
    for name, prec in (("mixed", T.CLBLM_PREC_MIXED), ("plain", T.CLBLM_PREC_PLAIN)):
        if name == "plain" and not fp64_jacobians:
            continue
        ctrl = T.rt_ctrl(precision=prec, grid_type=1)
        n, dv = h.jac_size(col, ctrl, prof)
        o = {key: torch.empty(shape, dtype=torch.float64, device="cuda")
             for key, shape in (("rad", n), ("dtlev", (nl + 1, n)), ("dqlev", (nl + 1, n)), ("dtsfc", n),
                                ("demis", n))}
        outs = [{k: v.data_ptr() for k, v in o.items()} | {"cap": n}]

        def call(graph=False):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            st = h.batch_device([col], ctrl, [prof], outs, graph=graph)
            torch.cuda.synchronize()
            assert st == [0], st
            return (time.perf_counter() - t0) * 1e3

        if name == "mixed":
            call()  # warm-up: workspace, tuning, the sticky JRAD settles
        ms = call()
        res["jacobians_" + name] = {"ms": ms, "points": n, "dv": dv, "value": n * nl / (ms * 1e-3), "unit": UNIT,
                                    "path": "clblm_gpu_batch, direct launches"}
        if name == "mixed":
            call(graph=True)  # capture
            reps = [call(graph=True) for _ in range(2)]
            res["jacobians_mixed_graph_replay"] = {"ms": min(reps), "value": n * nl / (min(reps) * 1e-3),
                                                   "unit": UNIT}
        jrad[name] = o["rad"]
        del o, outs
    if "plain" in jrad:
        m, p = jrad["mixed"], jrad["plain"]
        res["jacobian_leg_max_rel_rad_diff_mixed_vs_plain"] = float(((m - p).abs() / p.abs()).max())
        tm = res["radiance_mixed"]["ms"] + res["jacobians_mixed"]["ms"]
        tp = res["radiance_plain"]["ms"] + res["jacobians_plain"]["ms"]
        res["speedup_radiance_plus_jacobians_mixed_vs_plain"] = tp / tm
    del jrad
    h.close()
    torch.cuda.empty_cache()
    return res


def profile_case(args):
    """A bounded case for ncu captures of one kernel: the OD of one layer of the
    60-layer column over a narrower window (the full line list stays on the
    device: 20 MB; the layer's working set is a few hundred MB)."""
    import torch
    from clblm_gb300 import build as B
    from clblm_gb300 import capi, synth
    from clblm_gb300 import capi_types as T
    B.build()
    lines, col, cont = synth.config1()
    c = col.sub([args.profile_layer]).with_window(*args.window)
    dn, df, do = capi.setDV(c)
    g = T.grid_struct(c.v1, c.v2, dn[0], df[0])
    ctrl = T.od_ctrl(precision=T.CLBLM_PREC_PLAIN if args.plain else T.CLBLM_PREC_MIXED)
    h = capi.Handle(lines, cont)
    for _ in range(3):
        od, dv = h.odlay(c.layer(0), g, ctrl)
    torch.cuda.synchronize()
    st = h.stats()
    print("profile case: layer %d, %.1f-%.1f cm-1, %d points, dv %.3g, panel %.3f ms, f4 %.3f ms"
          % (args.profile_layer, c.v1, c.v2, len(od), dv, st["ms_panel"], st["ms_f4conv"]))
    h.close()


def profile_column(args):
    """A bounded radiance case for ncu captures: adjacent layers of the column
    over the full window."""
    import torch
    from clblm_gb300 import build as B
    from clblm_gb300 import capi, synth
    from clblm_gb300 import capi_types as T
    B.build()
    lines, col, cont = synth.config1()
    c = col.sub(list(range(*args.profile_column)))
    ctrl = T.rt_ctrl(precision=T.CLBLM_PREC_PLAIN if args.plain else T.CLBLM_PREC_MIXED)
    h = capi.Handle(lines, cont)
    for _ in range(2):
        rad, dv = h.rt_mode2(c, ctrl)
    torch.cuda.synchronize()
    st = h.stats()
    print("profile column: layers %d-%d, %d radiance points, %d launches per call"
          % (args.profile_column[0], args.profile_column[1] - 1, len(rad), st["launches"]))
    h.close()


def config_of(col, lines, lp, npts, world):
    """The workload's `config` object, the same in both arms."""
    return {"workload": WORKLOAD, "layers": col.nlay, "lines": lines.n, "layer_points_per_step": int(lp),
            "radiance_points": int(npts), "parallelism": "replicas" if world > 1 else "single GPU",
            "l2": "inputs larger than L2, no flush"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-plain", action="store_true", help="skip the FP64 GPU leg")
    ap.add_argument("--no-jac", action="store_true", help="skip the Jacobian leg (600-1100 cm-1)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-profiles leg (256 profiles)")
    ap.add_argument("--no-config4", action="store_true", help="skip the broadband leg (3 M lines, 100 layers)")
    ap.add_argument("--no-broadband-fp64-jacobians", action="store_true",
                    help="skip the FP64 timing of the broadband Jacobians (about 20 s)")
    ap.add_argument("--profile-layer", type=int, default=None,
                    help="profiling case: the OD of this one layer of the column, three calls, no JSON line")
    ap.add_argument("--window", type=float, nargs=2, default=(1000.0, 1200.0),
                    help="spectral window of the profiling case (cm-1)")
    ap.add_argument("--plain", action="store_true", help="profiling case in FP64")
    ap.add_argument("--profile-column", type=int, nargs=2, default=None, metavar=("FIRST", "LAST"),
                    help="profiling case: the radiance of layers FIRST..LAST-1 of the column, two calls")
    args = ap.parse_args()
    if args.profile_layer is not None:
        profile_case(args)
        return
    if args.profile_column is not None:
        profile_column(args)
        return

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))

    from clblm_gb300 import synth
    from clblm_gb300 import capi_types as T

    lines, col, cont = synth.config1()
    ctrl = T.rt_ctrl(precision=T.CLBLM_PREC_MIXED)

    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import oracle as O
        O.build()
        threads = os.cpu_count() or 1
        pctrl = T.rt_ctrl(precision=T.CLBLM_PREC_PLAIN)
        lp = layer_points_host(col, ctrl)
        # each step: the reference path on the whole column, all host threads
        # (one warm-up step: the CPU path has no state to warm)
        for _ in range(min(args.warmup, 1)):
            run_cpu(lines, col, cont, pctrl, threads)
        times = []
        rad = None
        for _ in range(args.steps):
            _, dt, rad = run_cpu(lines, col, cont, pctrl, threads)
            times.append(dt)
        v = lp / float(np.mean(times))
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(times)),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded, workload distributions)",
                "config": config_of(col, lines, lp, len(rad), world),
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                 "sample": "the whole 60-layer column, 500-2500 cm-1, every step: layer ODs "
                                           "OpenMP-parallel over layers, the merge's per-point loops OpenMP-parallel"},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    from clblm_gb300 import build as B
    from clblm_gb300 import capi
    B.build()
    torch.cuda.set_device(0)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    h = capi.Handle(lines, cont, device=torch.cuda.current_device())
    npts, _ = h.rt_size(col, ctrl)
    lp = layer_points(h, col, ctrl)
    rad_dev = torch.empty(npts, dtype=torch.float64, device="cuda")
    stream = torch.cuda.ExternalStream(h.stream())

    def step_dev(c=ctrl):
        h.rt_mode2_device(col, c, rad_dev.data_ptr(), npts)

    # warm-up (first calls grow the workspace)
    for _ in range(max(3, args.warmup)):
        step_dev()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kt = {"ms_panel": 0.0, "ms_f4conv": 0.0, "ms_line_chain": 0.0, "ms_f4_chain": 0.0, "ms_rt": 0.0,
          "launches": 0}
    with Clocks() as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            step_dev()
            st = h.stats()  # host-side counters of the call just made (no device sync)
            for k in kt:
                kt[k] += st[k]
        ev1.record(stream)
        torch.cuda.synchronize()
    work = dict(h.stats(), layers=col.nlay)
    ms = max_over_ranks(ev0.elapsed_time(ev1) / args.steps, "cuda")
    value = replica_value(lp, world, ms)

    # e2e through the C-ABI with host buffers
    plines = pinned_lines(lines)
    rad_host = torch.empty(npts, dtype=torch.float64, pin_memory=True).numpy()
    h2d = plines.nbytes()
    d2h = npts * 8
    for _ in range(2):
        h.set_lines(plines)
        h.rt_mode2(col, ctrl, out=rad_host)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        h.set_lines(plines)
        h.rt_mode2(col, ctrl, out=rad_host)
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    e2e_value = lp * world / (e2e_ms * 1e-3)

    # FP64 GPU path
    plain = None
    if not args.no_plain:
        pctrl = T.rt_ctrl(precision=T.CLBLM_PREC_PLAIN)
        step_dev(pctrl)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step_dev(pctrl)
        e1.record(stream)
        torch.cuda.synchronize()
        pms = e0.elapsed_time(e1)
        plain = {"value": lp / (pms * 1e-3), "unit": UNIT, "ms_per_step": pms}
        # radiance agreement of the mixed path with the FP64 GPU path
        r64 = torch.empty_like(rad_dev)
        h.rt_mode2_device(col, pctrl, r64.data_ptr(), npts)
        step_dev()
        torch.cuda.synchronize()
        plain["max_rel_rad_diff_mixed_vs_plain"] = float(((rad_dev - r64).abs() / r64.abs()).max().item())

    cpu = None
    oracle_err = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as O
        O.build()
        threads = os.cpu_count() or 1
        pctrl = T.rt_ctrl(precision=T.CLBLM_PREC_PLAIN)
        _, dt_all, rad_ref = run_cpu(lines, col, cont, pctrl, threads)
        sub, dt1, _ = run_cpu(lines, col, cont, pctrl, 1, CPU_LAYERS)
        pts1 = layer_points_host(sub, ctrl)
        cpu = {"value": lp / dt_all, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "the whole 60-layer column, 500-2500 cm-1, once (%.1f s; layer ODs OpenMP-parallel over "
                         "layers, the merge's per-point loops OpenMP-parallel)" % dt_all,
               "single_core": {"value": pts1 / dt1, "unit": UNIT, "cores": 1,
                               "sample": "layers %d-%d of the column, full 500-2500 cm-1, one thread (%.1f s)"
                                         % (CPU_LAYERS[0], CPU_LAYERS[-1], dt1)}}
        # every radiance of this run against the FP64 oracle's, whole column
        oracle_err = {"mixed": rel_err(rad_dev.cpu().numpy(), rad_ref),
                      "plain_fp64": rel_err(r64.cpu().numpy(), rad_ref) if plain is not None else None,
                      "e2e_mixed": rel_err(rad_host, rad_ref),
                      "what": "max over the 5.5 M radiance points of |GPU - oracle| / |oracle|, whole column; "
                              "bounds 1e-4 (mixed) and 1e-8 (FP64)"}

    jacl = None
    if not args.no_jac:
        jacl = jacobian_leg(cont, max(1, min(args.steps, 3)))
        jacl["autograd"] = autograd_leg(cont, max(1, min(args.steps, 3)))
    batl = None
    if not args.no_batch:
        batl = batch_leg(cont, 1)
    c4 = None
    if not args.no_config4:
        c4 = config4_leg(2, fp64_jacobians=not args.no_broadband_fp64_jacobians)
    roof = roofline(work, kt, args.steps, ms, lp)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32 (mixed: FP32 line shape + Kahan, FP64 index math)",
                "data": "synthetic (seeded, workload distributions)",
                "config": config_of(col, lines, lp, npts, world),
                "max_rel_err_vs_oracle": oracle_err,
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                        "ms_per_step": e2e_ms},
                "plain_fp64": plain, "jacobians": jacl, "batched_profiles": batl, "broadband": c4, "cpu_baseline": cpu, "roofline": roof,
                "clocks": clk.summary(),
                "gpu_launches": int(kt["launches"]),
                # per step, from events on the library's two streams: the line chain
                # and the far-wing chain run side by side before the panel kernel
                "stages_ms": {"line_chain": kt["ms_line_chain"] / args.steps,
                              "far_wing_chain": kt["ms_f4_chain"] / args.steps,
                              "k_f4_conv": kt["ms_f4conv"] / args.steps, "k_panel": kt["ms_panel"] / args.steps,
                              "k_rt_segment": kt["ms_rt"] / args.steps}}
        print(json.dumps(line))
    h.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
