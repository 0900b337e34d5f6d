#!/usr/bin/env python3
"""Marching-cubes throughput on one GB300: cells/s and HBM roofline fraction.

Workload (one "step"): the full marching-cubes forward pipeline with duplicate
point merging -- classify, count + scan, generate -- on a 512^3 float32 field
(sum of 8 seeded isotropic Gaussian blobs on the unit cube, isovalue 0.5),
field resident in HBM.  The field (537 MB) is larger than L2 (129 MB), so no
flush is needed between steps.

Reported:
  value        cells/s over all ranks, device-timed (CUDA events, field in HBM),
               one frame at a time: each frame is one dax_gb300_mc_pipeline
               call (count + merged generate of the whole grid, its z-slabs
               overlapping inside the call), replayed from a CUDA graph
               captured once (--no-graph: direct calls); "frames" reports the
               direct calls, the frame with a host read of the sizes, and the
               two-call path one frame at a time and with --frames frames in
               flight (default 4, each with its own field copy and stream)
  e2e          the same metric through the C ABI from page-locked host memory: every
               step copies its whole field to the device, sizes, generates and
               copies the surface back to host memory; two steps in flight on
               their own streams and buffers
  roofline     dominant kernel (K1 point classification): algorithmic bytes
               4P read + P/8 written per launch over its CUDA-event time
  cpu_baseline the CPU implementation on a bounded z-slab sample of the same
               field (see "sample")
With --impl reference the reference's CPU implementation (the DaxToolkit
worklets compiled from source, OpenMP over all host threads; the C oracle
port where that library is absent) is timed on the same workload instead.

Multi-GPU (torchrun): every rank processes its own 512^3 grid (independent
grids, no collective on the data path): weak scaling, value = all ranks'
cells / max over ranks of the timed region.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MC cells/s & HBM roofline % at 512^3 fp32"


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=1000)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--size", type=int, default=512)
    p.add_argument("--frames", type=int, default=4,
                   help="frames in flight (one stream, scratch and output set each)")
    p.add_argument("--classify-blocks-per-sm", type=int, default=3,
                   help="per-SM block limit of the classification pass while frames are in "
                        "flight, leaving room for the other frames' passes (0 = no limit)")
    p.add_argument("--slabs", type=int, default=0,
                   help="slabs of the pipelined frame (1..16; 0 = the library default)")
    p.add_argument("--fused", action="store_true",
                   help="run the count pass as the fused classify + count launch "
                        "(dax_gb300_set_fused_count) instead of separate passes")
    p.add_argument("--no-graph", action="store_true",
                   help="time direct pipelined calls instead of a CUDA-graph replay of one")
    p.add_argument("--cpu-seconds", type=float, default=12.0,
                   help="target CPU time of the bounded CPU-baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the adjoint / batched / threshold / gradient measurements")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(t_ms, world, device="cpu"):
    """The slowest rank's timed-region length (every rank calls this; one
    MAX all-reduce when world > 1)."""
    if world <= 1:
        return t_ms
    import torch
    import torch.distributed as dist
    tt = torch.tensor([t_ms], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def weak_value(world, units_per_rank, steps, t_ms):
    """Whole-job throughput under weak scaling: every rank's units over the
    slowest rank's time."""
    return world * units_per_rank * steps / (t_ms / 1e3)


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dram_traffic(kernel, workload):
    """Per-launch DRAM bytes (read + write) recorded from an ncu capture."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 3 and not line.startswith("#") and parts[0] == kernel and parts[1] == workload:
            return float(parts[2])
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(field_host, dims, spacing, iso, target_s, kind_pref="reference", threads=None):
    """Times count + merged generate of the CPU implementation on the first kz
    z-planes of the field, kz chosen so the run takes about target_s."""
    import numpy as np
    import oracle
    O = None
    if kind_pref == "reference":
        try:
            O = oracle.Oracle("reference")
        except Exception:
            O = None
    if O is None:
        O = oracle.Oracle("port")
    cores = O.set_threads(threads or O.max_threads()) if O.kind == "reference" else 1
    nx, ny, nz = dims
    f3 = field_host.reshape(nz, ny, nx)

    def run(kz):
        sub = np.ascontiguousarray(f3[:kz]).ravel()
        g = oracle.make_grid((nx, ny, kz), spacing=spacing)
        t0 = time.perf_counter()
        count, _ = O.mc_count(g, sub, iso)
        O.mc_generate(g, sub, iso, count, merge=True)
        return time.perf_counter() - t0, (nx - 1) * (ny - 1) * (kz - 1)

    t, c = run(min(nz, 9))
    per_cell = t / c
    kz = int(min(nz, max(9, target_s / per_cell / ((nx - 1) * (ny - 1)) + 1)))
    t, c = run(kz)
    return {"value": c / t, "unit": "cells/s", "cores": cores,
            "kind": "reference" if O.kind == "reference" else "port",
            "sample": "first %d of %d z-planes of the same field (%dx%dx%d points), "
                      "count + merged generate" % (kz, nz, nx, ny, kz),
            "seconds": t}


def reference_parity(field_host, dims, spacing, iso, verts, conn):
    """The timed frames' merged surface against the CPU implementation
    (the reference's own worklets where they compiled) on the whole field,
    bit for bit; run after the timed region."""
    import numpy as np
    import oracle
    O, cores = _ref_oracle()
    g = oracle.make_grid(dims, spacing=spacing)
    count, _ = O.mc_count(g, field_host, iso)
    ref = O.mc_generate(g, field_host, iso, count, merge=True)
    c = conn.cpu().numpy()
    v = verts.cpu().numpy()
    topo = c.shape == ref["conn"].shape and bool(np.array_equal(c, ref["conn"]))
    pos = v.shape == ref["verts"].shape and bool(
        np.array_equal(v.view(np.uint32), ref["verts"].view(np.uint32)))
    return {"against": "reference" if O.kind == "reference" else "port",
            "what": "merged triangles and vertices of the whole %dx%dx%d field" % tuple(dims),
            "topology": topo, "positions_bits": pos,
            "triangles": int(ref["conn"].shape[0]), "merged_vertices": int(ref["verts"].shape[0])}


def fp64_error_statement(field_host, dims, spacing, iso, grid, field, verts, conn, scratch):
    """Error of the float32 surface and cell gradients against the FP64 twin
    of the reference (its worklets built with DAX_USE_DOUBLE_PRECISION, same
    float32 inputs): marching-cubes weights and positions over the whole
    field, CellGradient over a 32-plane z-slab through the middle."""
    import ctypes as C_
    import numpy as np
    import torch
    import oracle
    from oracle import fp64_error
    from daxtoolkit_gb300 import cont
    try:
        tw = oracle.Fp64Twin()
    except RuntimeError as e:
        return {"unavailable": str(e)}
    nx, ny, nz = dims
    g = oracle.make_grid(dims, spacing=spacing)
    r64 = tw.mc_generate(g, field_host, iso, merge=True)
    rec = cont.marching_cubes(grid, field, iso, merge=True, records=True)
    same = bool(np.array_equal(rec["conn"].cpu().numpy(), r64["conn"]))
    mc = fp64_error.mc_error_stats(rec["verts"].cpu().numpy(), rec["rec_weight"].cpu().numpy(),
                                   r64, (0, 0, 0), spacing, (0, 0, 0), dims)
    k0, kp = nz // 2 - 16, 33
    sub = np.ascontiguousarray(field_host.reshape(nz, ny, nx)[k0:k0 + kp]).ravel()
    sg = cont.UniformGrid((nx, ny, kp), spacing=spacing, extent_min=(0, 0, k0))
    g32 = cont.cell_gradient(sg, torch.from_numpy(sub).to(field.device)).cpu().numpy()
    og = oracle.make_grid((nx, ny, kp), spacing=spacing, extent_min=(0, 0, k0))
    gr = fp64_error.gradient_error_stats(g32, tw.cell_gradient(og, sub), sub, (0, 0, 0), spacing,
                                         (0, 0, k0), (nx, ny, kp))
    gr["sample"] = "cell planes %d..%d of the %d^3 grid" % (k0, k0 + kp - 2, nx)
    return {"against": "reference worklets built with DAX_USE_DOUBLE_PRECISION, same float32 "
                       "inputs", "unit_roundoff": 2.0 ** -24, "topology_equal": same,
            "marching_cubes": mc, "cell_gradient": gr}


def _ref_oracle(threads=None):
    import oracle
    try:
        O = oracle.Oracle("reference")
    except Exception:
        O = oracle.Oracle("port")
    cores = O.set_threads(threads or O.max_threads()) if O.kind == "reference" else 1
    return O, cores


def cpu_slice_baseline(dims, spacing, origin, normal, target_s):
    """The CPU implementation's SliceCount + merged SliceGenerate on the first
    kz z-planes of the grid, kz chosen so the run takes about target_s."""
    import oracle
    O, cores = _ref_oracle()
    nx, ny, nz = dims

    def run(kz):
        g = oracle.make_grid((nx, ny, kz), spacing=spacing)
        t0 = time.perf_counter()
        c = O.slice_count(g, origin, normal)
        O.slice_generate(g, origin, normal, c, True)
        return time.perf_counter() - t0, (nx - 1) * (ny - 1) * (kz - 1)

    t, c = run(min(nz, 9))
    kz = int(min(nz, max(9, target_s / (t / c) / ((nx - 1) * (ny - 1)) + 1)))
    t, c = run(kz)
    return {"value": c / t, "unit": "cells/s", "cores": cores,
            "kind": "reference" if O.kind == "reference" else "port",
            "sample": "first %d of %d z-planes of the %dx%dx%d grid, count + merged generate"
                      % (kz, nz, nx, ny, nz)}


def cpu_mt_baseline(dims, spacing, field_host, iso, target_s):
    """The CPU implementation's MarchingTetrahedraCount + merged Generate on the
    tetrahedra of the first kz cell layers (Tetrahedralize order), kz chosen
    so the run takes about target_s."""
    import numpy as np
    import oracle
    O, cores = _ref_oracle()
    nx, ny, nz = dims
    f3 = field_host.reshape(nz, ny, nx)

    def run(kz):
        g = oracle.make_grid((nx, ny, kz + 1), spacing=spacing)
        conn = O.tetrahedralize(g)
        ax = [np.float32(spacing[a]) * np.arange(d, dtype=np.float32)
              for a, d in enumerate((nx, ny, kz + 1))]
        z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
        pts = np.stack([x.ravel(), y.ravel(), z.ravel()], 1)
        sub = np.ascontiguousarray(f3[:kz + 1]).ravel()
        t0 = time.perf_counter()
        c = O.mt_count(conn, sub, iso)
        O.mt_generate(pts, conn, sub, iso, c, True)
        return time.perf_counter() - t0, conn.shape[0]

    t, c = run(4)
    kz = int(min(nz - 1, max(4, target_s / (t / c) / (5 * (nx - 1) * (ny - 1)))))
    t, c = run(kz)
    return {"value": c / t, "unit": "tetrahedra/s", "cores": cores,
            "kind": "reference" if O.kind == "reference" else "port",
            "sample": "tetrahedra of the first %d of %d cell layers (%d), count + merged generate"
                      % (kz, nz - 1, c)}


def run_reference(args, rank, world):
    """The reference's CPU implementation on the host cores; rank 0 only."""
    if rank != 0:
        return
    import numpy as np
    import torch
    from daxtoolkit_gb300 import synthetic
    n = args.size
    dims = (n, n, n)
    spacing = (1.0 / (n - 1),) * 3
    field = synthetic.blob_field(dims, 8, seed=20260101, device="cpu").numpy()
    per_step = max(1.0, args.cpu_seconds / max(1, args.steps))
    for _ in range(args.warmup):
        cpu_baseline(field, dims, spacing, 0.5, min(per_step, 2.0))
    vals = [cpu_baseline(field, dims, spacing, 0.5, per_step) for _ in range(args.steps)]
    v = statistics.median([x["value"] for x in vals])
    C = (n - 1) ** 3
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "cells/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * C / v,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": config_dict(n),
        "cpu_baseline": {"value": v, "unit": "cells/s", "cores": vals[0]["cores"],
                         "kind": vals[0]["kind"], "sample": vals[0]["sample"]},
        "e2e": {"value": v, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _event_ms(fn, reps, stream):
    import torch
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fn()
    torch.cuda.synchronize()
    a.record(stream)
    for _ in range(reps):
        fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def extra_measurements(field, grid, dims, iso, peak, stream, dev, reps=50):
    """The rest of the headline metric: forward+adjoint against forward on the
    same 512^3 field; the 64-grid batched pipeline (one CUDA-graph replay)
    against the plain per-grid loop; threshold [0.3, 0.7] and CellGradient.
    All device-timed with CUDA events (the plain loop and the batched replay
    include the host read of the output sizes each iteration, which a caller
    needs to use the result)."""
    import torch
    from daxtoolkit_gb300 import capi, cont, synthetic
    L = capi.lib()
    s = ctypes.c_void_p(stream.cuda_stream)
    ptr = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
    g = grid.desc()
    nx, ny, nz = dims
    P, C = nx * ny * nz, (nx - 1) * (ny - 1) * (nz - 1)
    out = {}

    # --- forward (merged MC + CellGradient) vs forward + adjoint -----------
    nbytes = L.dax_gb300_mc_scratch_bytes(ctypes.byref(g))
    scratch = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    capi.call("dax_gb300_mc_count", ctypes.byref(g), ptr(field), iso, ptr(scratch), nbytes, s)
    T, V = ctypes.c_int64(0), ctypes.c_int64(0)
    capi.call("dax_gb300_mc_totals", ptr(scratch), ctypes.byref(T), ctypes.byref(V), s)
    T, V = T.value, V.value
    verts = torch.empty((V, 3), dtype=torch.float32, device=dev)
    conn = torch.empty((T, 3), dtype=torch.int32, device=dev)
    grad = torch.empty((C, 3), dtype=torch.float32, device=dev)
    dverts = torch.randn((V, 3), dtype=torch.float32, device=dev)
    dgrad = torch.randn((C, 3), dtype=torch.float32, device=dev)
    dfield = torch.empty_like(field)

    def fwd():
        capi.call("dax_gb300_mc_count", ctypes.byref(g), ptr(field), iso, ptr(scratch), nbytes, s)
        capi.call("dax_gb300_mc_generate", ctypes.byref(g), ptr(field), iso, 1, ptr(scratch),
                  nbytes, ptr(verts), V, ptr(conn), T, None, None, None, s)
        capi.call("dax_gb300_cell_gradient", ctypes.byref(g), ptr(field), ptr(grad), s)

    def bwd():  # recomputes the count pass instead of keeping it
        capi.call("dax_gb300_mc_count", ctypes.byref(g), ptr(field), iso, ptr(scratch), nbytes, s)
        capi.call("dax_gb300_field_adjoint", ctypes.byref(g), ptr(field), iso, ptr(scratch), nbytes,
                  ptr(dverts), ptr(dgrad), ptr(dfield), s)

    t_f = _event_ms(fwd, reps, stream)
    t_fb = _event_ms(lambda: (fwd(), bwd()), reps, stream)
    out["adjoint"] = {"workload": "merged MC + CellGradient forward, adjoint of both, %d^3" % nx,
                      "fwd_ms": t_f, "fwd_adj_ms": t_fb, "ratio": t_fb / t_f, "target_ratio": 3.0}

    # --- CellGradient and threshold ----------------------------------------
    t_g = _event_ms(lambda: capi.call("dax_gb300_cell_gradient", ctypes.byref(g), ptr(field),
                                      ptr(grad), s), reps, stream)
    gb = (4 * P + 12 * C) / (t_g / 1e3) / 1e9
    out["cell_gradient"] = {"ms": t_g, "cells_per_s": C / (t_g / 1e3), "achieved_gbs": gb,
                            "frac": gb / peak, "algorithmic_bytes": 4 * P + 12 * C}
    tb = L.dax_gb300_threshold_scratch_bytes(ctypes.byref(g))
    tscr = torch.empty(tb, dtype=torch.uint8, device=dev)
    capi.call("dax_gb300_threshold_count", ctypes.byref(g), ptr(field), 0.3, 0.7, ptr(tscr), tb, s)
    K, U = ctypes.c_int64(0), ctypes.c_int64(0)
    capi.call("dax_gb300_threshold_totals", ptr(tscr), ctypes.byref(K), ctypes.byref(U), s)
    K, U = K.value, U.value
    tconn = torch.empty((K, 8), dtype=torch.int32, device=dev)
    tcoords = torch.empty((U, 3), dtype=torch.float32, device=dev)
    tfield = torch.empty(U, dtype=torch.float32, device=dev)

    def thr():
        capi.call("dax_gb300_threshold_count", ctypes.byref(g), ptr(field), 0.3, 0.7, ptr(tscr), tb, s)
        capi.call("dax_gb300_threshold_generate", ctypes.byref(g), ptr(field), 0.3, 0.7, ptr(tscr),
                  tb, ptr(tconn), K, ptr(tcoords), ptr(tfield), U, s)

    t_t = _event_ms(thr, reps, stream)
    tbytes = 4 * P + 32 * K + 16 * U
    out["threshold"] = {"range": [0.3, 0.7], "kept_cells": K, "used_points": U, "ms": t_t,
                        "cells_per_s": C / (t_t / 1e3),
                        "achieved_gbs": tbytes / (t_t / 1e3) / 1e9,
                        "frac": tbytes / (t_t / 1e3) / 1e9 / peak,
                        "algorithmic_bytes": tbytes, "formula": "4P + 32K + 16U"}
    del scratch, tscr, grad, dgrad, dfield, tconn, tcoords, tfield

    # --- Slice: oblique plane through the same grid (fused, no field) ----
    po = (ctypes.c_float * 3)(0.45, 0.5, 0.55)
    pn = (ctypes.c_float * 3)(0.3, 0.9, -0.3)
    sscr = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    capi.call("dax_gb300_slice_count", ctypes.byref(g), po, pn, ptr(sscr), nbytes, s)
    ST, SV = ctypes.c_int64(0), ctypes.c_int64(0)
    capi.call("dax_gb300_mc_totals", ptr(sscr), ctypes.byref(ST), ctypes.byref(SV), s)
    ST, SV = ST.value, SV.value
    sverts = torch.empty((SV, 3), dtype=torch.float32, device=dev)
    sconn = torch.empty((ST, 3), dtype=torch.int32, device=dev)
    sfield = torch.empty_like(field)

    def slice_all():
        capi.call("dax_gb300_slice_count", ctypes.byref(g), po, pn, ptr(sscr), nbytes, s)
        capi.call("dax_gb300_slice_generate", ctypes.byref(g), po, pn, 1, ptr(sscr), nbytes,
                  ptr(sverts), SV, ptr(sconn), ST, None, None, None, s)

    def slice_field():
        capi.call("dax_gb300_slice_field", ctypes.byref(g), po, pn, ptr(sfield), None, s)

    t_s = _event_ms(slice_all, reps, stream)
    t_sf = _event_ms(slice_field, reps, stream)
    sbytes = P // 8 + 12 * SV + 12 * ST
    out["slice"] = {"plane": "origin (0.45,0.5,0.55), normal (0.3,0.9,-0.3), merged",
                    "triangles": ST, "points": SV, "ms": t_s, "cells_per_s": C / (t_s / 1e3),
                    "algorithmic_bytes": sbytes, "formula": "P/8 + 12V + 12T (no field stored)",
                    "achieved_gbs": sbytes / (t_s / 1e3) / 1e9,
                    "field_kernel_ms": t_sf, "field_kernel_gbs": 4 * P / (t_sf / 1e3) / 1e9,
                    "field_kernel_frac": 4 * P / (t_sf / 1e3) / 1e9 / peak}
    del sfield, sscr, sverts, sconn
    out["marching_tetrahedra"] = mt_measurements(peak, stream, dev, reps=max(3, reps // 5))
    out["mandelbulb"] = mandelbulb_measurements(stream, reps=max(3, reps // 5))
    out["reference_mc_benchmark"] = reference_benchmark_measurements(stream, reps=max(3, reps // 5))

    # --- 64 uneven grids: batched graph replay vs per-grid loop -------------
    gdims = synthetic.batch_grid_dims(64, 32, 192, 777)
    isos = synthetic.batch_isovalues(64, 0.3, 0.6, 777)
    grids, fields = [], []
    for k, d in enumerate(gdims):
        grids.append(cont.UniformGrid(d, spacing=tuple(1.0 / (x - 1) for x in d)))
        fields.append(synthetic.blob_field(d, 4, seed=1000 + k, noise=0.05, device=dev))
    cells = sum((d[0] - 1) * (d[1] - 1) * (d[2] - 1) for d in gdims)

    def plain():
        for gr, f, v in zip(grids, fields, isos):
            cont.marching_cubes(gr, f, v, merge=True)

    batch = cont.MarchingCubesBatch(grids, fields, isos)
    bv, bc, toff, voff = batch.run(merge=True)
    gv = torch.empty_like(bv)
    gc = torch.empty_like(bc)
    tuned = batch.autotune(gv, gc, merge=True)
    batch.capture(gv, gc, merge=True)

    def batched():
        batch.replay()
        batch.totals()

    t_plain = _event_ms(plain, 5, stream)
    t_batch = _event_ms(batched, 20, stream)
    t_batch_only = _event_ms(batch.replay, 20, stream)
    ok = bool(torch.equal(gv, bv) and torch.equal(gc, bc))

    # The plain kernels without the host in the loop: per grid
    # dax_gb300_mc_count + dax_gb300_mc_generate into outputs allocated
    # beforehand (each grid's own scratch, its exact sizes known from the
    # batch run), no size read between grids; as direct calls, and captured
    # once in a CUDA graph and replayed.
    gsl = []
    for k, (gr, f, v) in enumerate(zip(grids, fields, isos)):
        d = gr.desc()
        nb = L.dax_gb300_mc_scratch_bytes(ctypes.byref(d))
        T_k, V_k = toff[k + 1] - toff[k], voff[k + 1] - voff[k]
        gsl.append(dict(d=d, f=f, iso=float(v), nb=nb,
                        scr=torch.empty(nb, dtype=torch.uint8, device=dev),
                        verts=torch.empty((max(V_k, 1), 3), dtype=torch.float32, device=dev),
                        conn=torch.empty((max(T_k, 1), 3), dtype=torch.int32, device=dev),
                        T=T_k, V=V_k))

    def plain_kernels(st=s):
        for q in gsl:
            capi.call("dax_gb300_mc_count", ctypes.byref(q["d"]), ptr(q["f"]), q["iso"],
                      ptr(q["scr"]), q["nb"], st)
            capi.call("dax_gb300_mc_generate", ctypes.byref(q["d"]), ptr(q["f"]), q["iso"], 1,
                      ptr(q["scr"]), q["nb"], ptr(q["verts"]), q["V"], ptr(q["conn"]), q["T"],
                      None, None, None, st)

    t_plain_kernels = _event_ms(plain_kernels, 10, stream)
    side = torch.cuda.Stream(device=dev)
    side.wait_stream(stream)
    pg = torch.cuda.CUDAGraph()
    with torch.cuda.graph(pg, stream=side, capture_error_mode="thread_local"):
        plain_kernels(ctypes.c_void_p(side.cuda_stream))
    torch.cuda.synchronize()
    t_plain_graph = _event_ms(pg.replay, 20, stream)
    for k, q in enumerate(gsl):  # the loop's surfaces are the batch's, grid by grid
        ok = ok and bool(torch.equal(q["conn"][:q["T"]], bc[toff[k]:toff[k + 1]]))
        ok = ok and bool(torch.equal(q["verts"][:q["V"]], bv[voff[k]:voff[k + 1]]))
    del pg, gsl
    out["batched"] = {"grids": 64, "grid_dims": "each U{32..192}, seed 777", "cells": cells,
                      "triangles": toff[-1],
                      "plain_loop_ms": t_plain, "batched_graph_ms": t_batch,
                      "speedup": t_plain / t_batch, "target_speedup": 3.0,
                      "plain_kernels_loop_ms": t_plain_kernels,
                      "plain_kernels_loop_graph_ms": t_plain_graph,
                      "batched_graph_replay_only_ms": t_batch_only,
                      "speedup_vs_plain_kernels_graph": t_plain_graph / t_batch_only,
                      "speedup_vs_plain_kernels_direct": t_plain_kernels / t_batch_only,
                      "batched_cells_per_s": cells / (t_batch / 1e3),
                      "autotuned": {"emit_batch": tuned[0], "dealt_count": tuned[1],
                                    "best_ms": tuned[2]},
                      "note": "plain_loop: cont.marching_cubes per grid (allocation and a host "
                              "size read per grid); plain_kernels: count + generate per grid into "
                              "preallocated outputs, no host read, direct or one graph replay; "
                              "batched_graph_replay_only: the batch's graph replay without the "
                              "totals read",
                      "graph_replay_matches_batch_run": ok}
    del grids, fields, batch, bv, bc, gv, gc
    out["batched_forward_adjoint"] = batch_adjoint_measurements(stream, dev)
    out["primitives"] = primitive_measurements(peak, stream, dev)
    return out


def batch_adjoint_measurements(stream, dev, reps=20):
    """32 grids, each dimension U{64..160}, 16 blobs, isovalue U[0.3,0.6]:
    forward (count, merged generate, CellGradient) and adjoint (the count
    pass again, dL/dfield from dL/dvertices and dL/dgradient) of every grid,
    (a) as the per-grid sequence of single-grid calls, (b) as the grid-set
    launches (one per pass for all grids), each captured in one CUDA graph
    and replayed.  The two arms' dL/dfield agree bit for bit."""
    import torch
    from daxtoolkit_gb300 import capi, cont, synthetic
    L = capi.lib()
    ptr = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
    dims = synthetic.batch_grid_dims(32, 64, 160, 1024)
    isos = synthetic.batch_isovalues(32, 0.3, 0.6, 1024)
    grids, fields = [], []
    for q, d in enumerate(dims):
        grids.append(cont.UniformGrid(d, spacing=tuple(1.0 / (x - 1) for x in d)))
        fields.append(synthetic.blob_field(d, 16, seed=3000 + q, device=dev))
    batch = cont.MarchingCubesBatch(grids, fields, isos)
    verts, conn, toff, voff = batch.run(merge=True)
    C, P = batch.sizes()
    grad = torch.empty((C, 3), dtype=torch.float32, device=dev)
    dV = torch.randn_like(verts)
    dG = torch.randn((C, 3), dtype=torch.float32, device=dev)
    dfield = torch.empty(P, dtype=torch.float32, device=dev)
    items, c0, p0 = [], 0, 0
    for q, (gr, f, iso) in enumerate(zip(grids, fields, isos)):
        d = gr.desc()
        nb = L.dax_gb300_mc_scratch_bytes(ctypes.byref(d))
        nc, npts = gr.GetNumberOfCells(), gr.GetNumberOfPoints()
        items.append(dict(d=d, f=f, iso=float(iso), nb=nb,
                          scr=torch.empty(nb, dtype=torch.uint8, device=dev),
                          verts=torch.empty((max(voff[q + 1] - voff[q], 1), 3), device=dev),
                          conn=torch.empty((max(toff[q + 1] - toff[q], 1), 3), dtype=torch.int32,
                                           device=dev),
                          V=voff[q + 1] - voff[q], T=toff[q + 1] - toff[q],
                          grad=grad[c0:c0 + nc], dV=dV[voff[q]:voff[q + 1]].contiguous(),
                          dG=dG[c0:c0 + nc], out=torch.empty(npts, device=dev), p0=p0))
        c0 += nc
        p0 += npts

    def per_grid(st):
        for it in items:
            d = ctypes.byref(it["d"])
            capi.call("dax_gb300_mc_count", d, ptr(it["f"]), it["iso"], ptr(it["scr"]), it["nb"], st)
            capi.call("dax_gb300_mc_generate", d, ptr(it["f"]), it["iso"], 1, ptr(it["scr"]),
                      it["nb"], ptr(it["verts"]), it["V"], ptr(it["conn"]), it["T"], None, None,
                      None, st)
            capi.call("dax_gb300_cell_gradient", d, ptr(it["f"]), ptr(it["grad"]), st)
            capi.call("dax_gb300_mc_count", d, ptr(it["f"]), it["iso"], ptr(it["scr"]), it["nb"], st)
            capi.call("dax_gb300_field_adjoint", d, ptr(it["f"]), it["iso"], ptr(it["scr"]),
                      it["nb"], ptr(it["dV"]), ptr(it["dG"]), ptr(it["out"]), st)

    def grid_set(st):
        batch.count(st)
        batch.generate(verts, conn, True, st)
        batch.cell_gradient(grad, st)
        batch.count(st)
        batch.field_adjoint(dV, dG, dfield, st)

    side = torch.cuda.Stream(device=dev)
    res = {}
    for name, fn in (("per_grid", per_grid), ("grid_set", grid_set)):
        side.wait_stream(stream)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side, capture_error_mode="thread_local"):
            fn(side)
        torch.cuda.synchronize()
        res[name] = _event_ms(g.replay, reps, stream)
        del g
    ok = all(bool(torch.equal(it["out"].view(torch.int32),
                              dfield[it["p0"]:it["p0"] + it["out"].numel()].view(torch.int32)))
             for it in items)
    return {"grids": 32, "grid_dims": "each U{64..160}, seed 1024",
            "cells": C, "points": P, "triangles": toff[-1],
            "per_grid_graph_ms": res["per_grid"], "grid_set_graph_ms": res["grid_set"],
            "speedup": res["per_grid"] / res["grid_set"],
            "grid_set_matches_per_grid": ok,
            "note": "forward (count, merged generate, CellGradient) + adjoint (count recomputed, "
                    "dL/dfield of vertices and gradients) of every grid, each arm one CUDA graph"}


def mt_measurements(peak, stream, dev, reps=10, n=256):
    """Marching tetrahedra on an n^3 grid split 5 ways by Tetrahedralize
    (83 M tetrahedra at n = 256), the 8-blob field, isovalue 0.5: the count
    pass alone (4 B id x 4 + 1 B case per tetrahedron, field gathers from
    L2), and count + generate unmerged and merged (sort / unique / bounds;
    the merged call reads T and V back to the host, as a caller must)."""
    import torch
    from daxtoolkit_gb300 import capi, cont, synthetic
    L = capi.lib()
    s = ctypes.c_void_p(stream.cuda_stream)
    ptr = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
    grid = cont.UniformGrid((n, n, n), spacing=(1.0 / (n - 1),) * 3)
    tg = cont.tetrahedralize(grid)
    conn, pts = tg.GetCellConnections(), tg.GetPointCoordinates()
    f = synthetic.blob_field((n, n, n), 8, seed=0, device=dev)
    C, P = conn.shape[0], pts.shape[0]
    iso = 0.5
    nb = L.dax_gb300_mt_scratch_bytes(C)
    scr = torch.empty(nb, dtype=torch.uint8, device=dev)

    def count():
        capi.call("dax_gb300_mt_count", ptr(conn), C, ptr(f), P, iso, ptr(scr), nb, s)

    t_count = _event_ms(count, reps, stream)
    t_unmerged = _event_ms(lambda: cont.marching_tetrahedra(tg, f, iso, merge=False, stream=stream),
                           reps, stream)
    t_merged = _event_ms(lambda: cont.marching_tetrahedra(tg, f, iso, merge=True, stream=stream),
                         reps, stream)
    o = cont.marching_tetrahedra(tg, f, iso, merge=True, stream=stream)
    cbytes = 17 * C
    return {"grid": "%d^3 points, Tetrahedralize (5 per voxel)" % n, "n": n, "tetrahedra": C,
            "triangles": int(o["conn"].shape[0]), "merged_points": int(o["verts"].shape[0]),
            "count_ms": t_count, "count_gbs": cbytes / (t_count / 1e3) / 1e9,
            "count_frac": cbytes / (t_count / 1e3) / 1e9 / peak,
            "count_formula": "17 B per tetrahedron (ids + case byte)",
            "unmerged_ms": t_unmerged, "merged_ms": t_merged,
            "tetrahedra_per_s_merged": C / (t_merged / 1e3)}


def reference_benchmark_measurements(stream, reps=10, sizes=(128, 256, 512)):
    """The reference's own marching-cubes benchmark workload
    (Benchmarks/MarchingCubes: main.cxx:21-44, Pipeline.h:100-150): a dim^3
    grid of unit spacing, Magnitude of the point coordinates, marching cubes
    at isovalue 100 with points merged (REMOVE_DUPLICATES) or not; the
    benchmark's default size is 128.  The time is the benchmark's timed
    region (count + generate, the field already computed), device-timed; the
    VTK dump of the 128^3 merged surface is timed on the host."""
    import tempfile
    from daxtoolkit_gb300 import cont
    out = {}
    for dim in sizes:
        grid = cont.UniformGrid((dim,) * 3)
        f = cont.point_magnitude(grid, stream=stream)
        C = grid.GetNumberOfCells()
        row = {"cells": C}
        for merge in (False, True):
            o = cont.marching_cubes(grid, f, 100.0, merge=merge, stream=stream)
            t = _event_ms(lambda: cont.marching_cubes(grid, f, 100.0, merge=merge, stream=stream),
                          reps, stream)
            key = "remove_duplicates" if merge else "plain"
            row[key] = {"ms": t, "cells_per_s": C / (t / 1e3), "triangles": int(o["conn"].shape[0]),
                        "points": int(o["verts"].shape[0])}
        out["dim%d" % dim] = row
        if dim == 128:
            o = cont.marching_cubes(grid, f, 100.0, merge=True, stream=stream)
            with tempfile.TemporaryDirectory() as d:
                path = d + "/MCdaxResult.vtk"
                t0 = time.perf_counter()
                cont.write_vtk(path, cont.UnstructuredGrid(o["verts"], o["conn"]))
                dt = time.perf_counter() - t0
                size = os.path.getsize(path)
            out["vtk_write_128"] = {"bytes": size, "seconds": dt, "mb_per_s": size / dt / 1e6}
    return out


def cpu_reference_benchmark(dim=128):
    """The reference's CPU implementation (its worklets built from source,
    OpenMP over all host threads) on the whole dim^3 benchmark workload."""
    import oracle
    O, cores = _ref_oracle()
    g = oracle.make_grid((dim,) * 3)
    f = O.point_magnitude(g)
    out = {"cores": cores, "kind": "reference" if O.kind == "reference" else "port",
           "sample": "the whole %d^3 benchmark grid" % dim, "unit": "cells/s"}
    for merge in (False, True):
        t0 = time.perf_counter()
        c, _ = O.mc_count(g, f, 100.0)
        O.mc_generate(g, f, 100.0, c, merge)
        dt = time.perf_counter() - t0
        out["remove_duplicates" if merge else "plain"] = (dim - 1) ** 3 / dt
    return out


def mandelbulb_measurements(stream, reps=10, sizes=(200, 512), iteration=3.5, cut=0.8):
    """The Mandelbulb benchmark's compute pipeline (computeMandlebulb,
    extractSurface, extractCut with ColorsAndNorms; Benchmarks/Mandlebulb) on
    its own volume -- origin -1, spacing 2/n, points 0..n -- at the demo's
    default n = 200 and at n = 512.  The escape-iteration field is bound by
    the transcendental functions of up to 34 iterations per point, not by
    memory; the surfaces are marching cubes of it."""
    from daxtoolkit_gb300 import cont
    out = {}
    for n in sizes:
        vol = cont.compute_mandlebulb((-1.0,) * 3, (2.0 / n,) * 3, (n, n, n), stream=stream)
        t_field = _event_ms(lambda: cont.mandlebulb_field(vol.Grid, stream=stream), reps, stream)
        surf = cont.extract_surface(vol, iteration, stream=stream)
        t_surf = _event_ms(lambda: cont.extract_surface(vol, iteration, stream=stream), reps, stream)
        cutsurf = cont.extract_cut(vol, cut, iteration, stream=stream)
        t_cut = _event_ms(lambda: cont.extract_cut(vol, cut, iteration, stream=stream), reps, stream)
        P = vol.Grid.GetNumberOfPoints()
        out["n%d" % n] = {"points": P, "field_ms": t_field, "points_per_s": P / (t_field / 1e3),
                          "iteration": iteration, "surface_triangles": surf.Data.GetNumberOfCells(),
                          "surface_ms": t_surf, "cut": cut,
                          "cut_triangles": cutsurf.Data.GetNumberOfCells(), "cut_ms": t_cut}
    return out


def cpu_mandelbulb_baseline(n, target_s):
    """The C restatement of the Mandelbulb escape iteration (single thread; the
    reference's worklet needs Boost.Preprocessor and is not built here) on the
    first kz z-planes of the n^3 volume, kz chosen so it takes about target_s."""
    import oracle
    O = oracle.Oracle("port")
    sp = 2.0 / n

    def run(kz):
        g = oracle.make_grid((n + 1, n + 1, kz), (-1.0, -1.0, -1.0 + sp * (n // 2)), (sp,) * 3)
        t0 = time.perf_counter()
        O.mandelbulb_field(g)
        return time.perf_counter() - t0, (n + 1) * (n + 1) * kz

    t, c = run(2)
    kz = int(min(n + 1 - n // 2, max(2, target_s / (t / c) / ((n + 1) ** 2))))
    t, c = run(kz)
    return {"value": c / t, "unit": "points/s", "cores": 1, "kind": "port",
            "sample": "escape iteration of %d z-planes through the middle of the %d^3-cell volume"
                      % (kz, n)}


def primitive_measurements(peak, stream, dev, reps=10):
    """The device adapter's generic primitives on large int32 inputs, device-
    timed, with numpy on the host cores beside them (the reference's CPU
    adapter runs std:: algorithms of the same kind).  Bytes per element are
    the data each algorithm must touch at least once."""
    import numpy as np
    import torch
    from daxtoolkit_gb300 import cont
    A = cont.Algorithm
    g = torch.Generator(device="cpu").manual_seed(4321)
    res = {}

    def gbs(nbytes, ms):
        return nbytes / (ms / 1e3) / 1e9

    def cpu_ms(fn, k=3):
        t0 = time.perf_counter()
        for _ in range(k):
            fn()
        return (time.perf_counter() - t0) / k * 1e3

    # ScanInclusive over 1 G dax::Id values (read 4 B, write 4 B)
    n = 1 << 30
    x = torch.randint(0, 1000, (n,), dtype=torch.int32, device=dev)
    y = torch.empty_like(x)
    t = _event_ms(lambda: A.ScanInclusive(x, y), reps, stream)
    xs = x[: 1 << 26].cpu().numpy()
    tc = cpu_ms(lambda: np.cumsum(xs, dtype=np.int32)) * (n / (1 << 26))
    res["scan_inclusive_i32"] = {"n": n, "ms": t, "gb_s": gbs(8 * n, t), "frac": gbs(8 * n, t) / peak,
                                 "cpu_numpy_ms_scaled": tc}
    del x, y
    # SortByKey of 100 M (int32 key, int32 value) pairs (read and write 8 B)
    n = 100_000_000
    keys0 = torch.randint(-2 ** 31, 2 ** 31 - 1, (n,), dtype=torch.int32, generator=g).to(dev)
    vals0 = torch.arange(n, dtype=torch.int32, device=dev)
    keys, vals = keys0.clone(), vals0.clone()

    def sort_once():
        keys.copy_(keys0)
        vals.copy_(vals0)
        A.SortByKey(keys, vals)

    t_copy = _event_ms(lambda: (keys.copy_(keys0), vals.copy_(vals0)), reps, stream)
    t = _event_ms(sort_once, reps, stream) - t_copy
    ok = bool(torch.all(keys[1:] >= keys[:-1]).item())
    kc = keys0[: 1 << 24].cpu().numpy()
    tc = cpu_ms(lambda: np.argsort(kc, kind="stable")) * (n / (1 << 24))
    res["sort_by_key_i32_pairs"] = {"n": n, "ms": t, "keys_per_s": n / (t / 1e3),
                                    "gb_s_min_traffic": gbs(16 * n, t), "sorted": ok,
                                    "passes": 4, "cpu_numpy_stable_argsort_ms_scaled": tc}
    # Unique of the sorted keys, StreamCompact of the values with a 30 % stencil
    uk = keys.clone()
    t_u = _event_ms(lambda: (uk.copy_(keys), A.Unique(uk)), reps, stream) - \
        _event_ms(lambda: uk.copy_(keys), reps, stream)
    stencil = (torch.rand(n, generator=g) < 0.3).to(torch.int32).to(dev)
    t_c = _event_ms(lambda: A.StreamCompact(vals, stencil), reps, stream)
    res["unique_i32"] = {"n": n, "ms": t_u, "gb_s_min_traffic": gbs(8 * n, t_u)}
    res["stream_compact_i32"] = {"n": n, "kept": int(stencil.sum().item()), "ms": t_c,
                                 "gb_s_min_traffic": gbs(8 * n + 4 * int(stencil.sum().item()), t_c)}
    return res


def config_dict(n):
    return {"workload": "marching cubes forward, %d^3 points float32, 8 gaussian blobs "
                        "(seed 20260101), isovalue 0.5, duplicate-point merge on" % n,
            "grid_points": [n, n, n], "isovalue": 0.5, "merge": True,
            "l2_policy": "inputs larger than L2 (field %d MB > 129 MB), no flush" %
                         (4 * n ** 3 // 2 ** 20)}


def main():
    args = parse_args()
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "gb300" else "gloo"
        if args.impl == "gb300":
            import torch
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    if args.impl == "reference":
        run_reference(args, rank, world)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    import numpy as np
    import torch

    from daxtoolkit_gb300 import build as gbuild
    gbuild.build()
    from daxtoolkit_gb300 import capi, cont, synthetic

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n = args.size
    dims = (n, n, n)
    spacing = (1.0 / (n - 1),) * 3
    iso = 0.5
    P, C = n ** 3, (n - 1) ** 3
    field = synthetic.blob_field(dims, 8, seed=20260101, device=dev)
    grid = cont.UniformGrid(dims, spacing=spacing)
    g = grid.desc()
    L = capi.lib()
    stream = torch.cuda.current_stream()
    s = ctypes.c_void_p(stream.cuda_stream)
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())
    nbytes = L.dax_gb300_mc_scratch_bytes(ctypes.byref(g))
    scratch = torch.empty(nbytes, dtype=torch.uint8, device=dev)

    # size outputs once (the count is deterministic for a fixed field)
    capi.call("dax_gb300_mc_count", ctypes.byref(g), ptr(field), iso, ptr(scratch), nbytes, s)
    T, V = ctypes.c_int64(0), ctypes.c_int64(0)
    capi.call("dax_gb300_mc_totals", ptr(scratch), ctypes.byref(T), ctypes.byref(V), s)
    T, V = T.value, V.value
    verts = torch.empty((V, 3), dtype=torch.float32, device=dev)
    conn = torch.empty((T, 3), dtype=torch.int32, device=dev)

    # The headline frame: dax_gb300_mc_pipeline, one complete count +
    # generate of the whole grid per call (its slabs overlap inside the
    # call), one frame at a time: each frame's passes are all queued on the
    # stream after the previous frame's have finished, so nothing of two
    # frames overlaps.  The frame's calls are captured once in a CUDA graph
    # and replayed (the same kernels, without the host enqueue cost of the
    # slab launches); --no-graph times the direct calls.
    capi.call("dax_gb300_set_pipeline_slabs", args.slabs)
    capi.call("dax_gb300_set_fused_count", 1 if args.fused else 0, 0)
    plan = (ctypes.c_int64 * 52)()
    capi.call("dax_gb300_mc_pipeline_plan", ctypes.byref(g), 0, plan)
    slab_count = int(plan[0])

    def pipe_frame(st=s):
        capi.call("dax_gb300_mc_pipeline", ctypes.byref(g), ptr(field), iso, 1, ptr(scratch),
                  nbytes, ptr(verts), V, ptr(conn), T, None, None, None, st)

    pipe_frame()
    torch.cuda.synchronize()
    graph = None
    if not args.no_graph:
        side = torch.cuda.Stream(device=dev)
        side.wait_stream(stream)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=side, capture_error_mode="thread_local"):
            pipe_frame(ctypes.c_void_p(side.cuda_stream))
        torch.cuda.synchronize()

    def frame():
        if graph is not None:
            graph.replay()
        else:
            pipe_frame()

    def run_timed(count, fn):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(count):
            fn()
        b.record(stream)
        return a, b

    for _ in range(max(3, args.warmup)):
        frame()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    barrier()
    torch.cuda.synchronize()
    e0, e1 = run_timed(args.steps, frame)
    torch.cuda.synchronize()
    barrier()
    t_ms = e0.elapsed_time(e1)
    clocks = sampler.stop()
    T2, V2 = ctypes.c_int64(0), ctypes.c_int64(0)
    capi.call("dax_gb300_mc_totals", ptr(scratch), ctypes.byref(T2), ctypes.byref(V2), s)
    assert (T2.value, V2.value) == (T, V)
    verts_pipe, conn_pipe = verts.clone(), conn.clone()
    t_ms = max_over_ranks(t_ms, world, dev)
    ms_per_step = t_ms / args.steps
    value = weak_value(world, C, args.steps, t_ms)
    reps1 = max(5, min(args.steps, 300))

    def timed_frames(count, fn):
        fn()
        torch.cuda.synchronize()
        a, b = run_timed(count, fn)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / count

    # the same pipelined frame, direct calls (no graph), and with the host
    # reading the sizes after every frame (the reference's timer window
    # holds its one host sync, Benchmarks/MarchingCubes/Pipeline.h:110-132)
    ms_direct = timed_frames(reps1, pipe_frame)

    def frame_and_sizes():
        frame()
        Tq, Vq = ctypes.c_int64(0), ctypes.c_int64(0)
        capi.call("dax_gb300_mc_totals", ptr(scratch), ctypes.byref(Tq), ctypes.byref(Vq), s)

    ms_with_sizes = timed_frames(reps1, frame_and_sizes)

    # The two-call path (dax_gb300_mc_count, then dax_gb300_mc_generate), one
    # frame at a time, and with --frames frames in flight: consecutive frames
    # go to separate streams, each with its own copy of the field, scratch and
    # outputs, so one frame's classification overlaps the count, scan and
    # emit of the frames before it.
    F = max(1, args.frames)
    slots = []
    for f in range(F):
        slots.append(dict(
            field=field if f == 0 else field.clone(),
            scratch=scratch if f == 0 else torch.empty_like(scratch),
            verts=verts if f == 0 else torch.empty_like(verts),
            conn=conn if f == 0 else torch.empty_like(conn),
            stream=torch.cuda.Stream(device=dev)))
    for sl in slots:
        sl["s"] = ctypes.c_void_p(sl["stream"].cuda_stream)

    def two_call_frame(k, inflight):
        sl = slots[k % inflight]
        capi.call("dax_gb300_mc_count", ctypes.byref(g), ptr(sl["field"]), iso, ptr(sl["scratch"]),
                  nbytes, sl["s"])
        capi.call("dax_gb300_mc_generate", ctypes.byref(g), ptr(sl["field"]), iso, 1,
                  ptr(sl["scratch"]), nbytes, ptr(sl["verts"]), V, ptr(sl["conn"]), T, None, None,
                  None, sl["s"])

    def run_frames(count, inflight):
        cur = torch.cuda.current_stream()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(cur)
        for sl in slots:
            sl["stream"].wait_stream(cur)
        for k in range(count):
            two_call_frame(k, inflight)
        for sl in slots:
            cur.wait_stream(sl["stream"])
        b.record(cur)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / count

    run_frames(2, 1)
    ms_one = run_frames(reps1, 1)
    capi.call("dax_gb300_set_blocks_per_sm", 0, max(0, args.classify_blocks_per_sm))
    run_frames(3 * F, F)
    ms_inflight = run_frames(reps1, F)
    capi.call("dax_gb300_set_blocks_per_sm", 0, 0)
    for sl in slots:
        T3, V3 = ctypes.c_int64(0), ctypes.c_int64(0)
        capi.call("dax_gb300_mc_totals", ptr(sl["scratch"]), ctypes.byref(T3), ctypes.byref(V3),
                  sl["s"])
        assert (T3.value, V3.value) == (T, V)
        assert torch.equal(sl["verts"], verts_pipe) and torch.equal(sl["conn"], conn_pipe)
    del slots

    # --- per-stage timing: K1 alone, count pass, generate pass -------------
    bits = torch.empty(L.dax_gb300_classify_words(P), dtype=torch.int32, device=dev)

    def timed(fn, reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    reps = max(5, min(args.steps, 200))
    k1 = lambda: capi.call("dax_gb300_classify_points", ptr(field), P, 0, iso, 0.0, ptr(bits), s)
    k1()
    t_k1 = timed(k1, reps)
    t_count = timed(lambda: capi.call("dax_gb300_mc_count", ctypes.byref(g), ptr(field), iso,
                                      ptr(scratch), nbytes, s), reps)
    t_gen = timed(lambda: capi.call("dax_gb300_mc_generate", ctypes.byref(g), ptr(field), iso, 1,
                                    ptr(scratch), nbytes, ptr(verts), V, ptr(conn), T, None, None,
                                    None, s), reps)

    peak, peak_kind = measured_peaks()
    k1_bytes = 4 * P + P / 8
    achieved = k1_bytes / (t_k1 / 1e3) / 1e9
    traffic = dram_traffic("k_classify_bits", "%dcube" % n)
    alg_bytes = 4 * P + 12 * V + 12 * T
    pipe_gbs = alg_bytes / (ms_per_step / 1e3) / 1e9

    # --- end to end through the public API, host buffers ------------------
    # End to end through the C ABI from page-locked host memory: every step
    # copies its whole 512^3 field from page-locked host memory to the device,
    # sizes its outputs from the totals, generates and copies the surface back
    # to page-locked host memory.  Two steps are in flight on their own
    # streams, each with its own host field, device copy, scratch and outputs:
    # step k+1's field crosses the host link while step k sizes, generates and
    # copies its surface out the other way.
    E = 2
    hf0 = field.cpu()
    eslots = []
    for q in range(E):
        hf = torch.empty(P, dtype=torch.float32, pin_memory=True)
        hf.copy_(hf0)
        eslots.append(dict(
            host=hf, dfield=torch.empty(P, dtype=torch.float32, device=dev),
            scratch=torch.empty(nbytes, dtype=torch.uint8, device=dev),
            verts=torch.empty((V, 3), dtype=torch.float32, device=dev),
            conn=torch.empty((T, 3), dtype=torch.int32, device=dev),
            hv=torch.empty((V, 3), dtype=torch.float32, pin_memory=True),
            hc=torch.empty((T, 3), dtype=torch.int32, pin_memory=True),
            stream=torch.cuda.Stream(device=dev)))
    for q in eslots:
        q["s"] = ctypes.c_void_p(q["stream"].cuda_stream)
        q["aux"] = torch.cuda.Stream(device=dev)
        q["copied"] = torch.cuda.Event()
    del hf0
    # A step's field crosses the host link as two halves on two streams: one
    # copy alone moves about half of what two concurrent ones move, and the
    # steps' own copies overlap only some of the time.
    half = (P // 2) & ~1023

    def copy_field(q):
        q["aux"].wait_stream(q["stream"])  # the slot's last generate has read the field
        with torch.cuda.stream(q["aux"]):
            q["dfield"][half:].copy_(q["host"][half:], non_blocking=True)
            q["copied"].record(q["aux"])
        with torch.cuda.stream(q["stream"]):
            q["dfield"][:half].copy_(q["host"][:half], non_blocking=True)
            q["stream"].wait_event(q["copied"])

    def e2e_count(q):
        copy_field(q)
        capi.call("dax_gb300_mc_count", ctypes.byref(g), ptr(q["dfield"]), iso, ptr(q["scratch"]),
                  nbytes, q["s"])

    def e2e_finish(q):
        Tq, Vq = ctypes.c_int64(0), ctypes.c_int64(0)
        capi.call("dax_gb300_mc_totals", ptr(q["scratch"]), ctypes.byref(Tq), ctypes.byref(Vq),
                  q["s"])
        assert (Tq.value, Vq.value) == (T, V)
        capi.call("dax_gb300_mc_generate", ctypes.byref(g), ptr(q["dfield"]), iso, 1,
                  ptr(q["scratch"]), nbytes, ptr(q["verts"]), Vq.value, ptr(q["conn"]), Tq.value,
                  None, None, None, q["s"])
        with torch.cuda.stream(q["stream"]):
            q["hv"].copy_(q["verts"], non_blocking=True)
            q["hc"].copy_(q["conn"], non_blocking=True)

    def e2e_run(steps):
        pending = None
        for k in range(steps):
            q = eslots[k % E]
            e2e_count(q)               # enqueued before the host waits on the previous step
            if pending is not None:
                e2e_finish(pending)
            pending = q
        e2e_finish(pending)
        for q in eslots:
            q["stream"].synchronize()

    e2e_steps = max(3, min(args.steps, 50))
    e2e_run(2 * E)
    barrier()
    t0 = time.perf_counter()
    e2e_run(e2e_steps)
    barrier()
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    for q in eslots:
        assert torch.equal(q["hv"], verts.cpu()) and torch.equal(q["hc"], conn.cpu())
    e2e_value = world * C / t_e2e

    # The floor e2e is held to: the fields' host-to-device copies alone, from
    # the same page-locked buffers, split and in flight as in the e2e steps.
    def h2d_round():
        for q in eslots:
            copy_field(q)

    h2d_round()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(5):
        h2d_round()
    torch.cuda.synchronize()
    h2d_ms = (time.perf_counter() - t0) / (5 * E) * 1e3
    h2d_gbs = 4 * P / (h2d_ms / 1e3) / 1e9

    line = {
        "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": dict(config_dict(n), frames_in_flight=1, slabs=slab_count,
                       call="dax_gb300_mc_pipeline (count + merged generate, slab-pipelined)",
                       count_pass="fused classify + count launch, then the scan" if args.fused
                       else "classification, staged count and scan launches",
                       replay="CUDA graph of the frame's call, captured once" if graph is not None
                       else "direct call per frame"),
        "frames": {"pipelined_direct_calls_ms": ms_direct,
                   "pipelined_with_host_size_read_ms": ms_with_sizes,
                   "two_call_one_at_a_time_ms": ms_one,
                   "two_call_in_flight_ms": ms_inflight, "two_call_frames_in_flight": F,
                   "two_call_classify_blocks_per_sm_in_flight": args.classify_blocks_per_sm,
                   "note": "ms per frame; 'in flight' frames each have their own field copy, "
                           "scratch, outputs and stream"},
        "triangles": T, "merged_vertices": V,
        "triangles_per_s": world * T / (ms_per_step / 1e3),
        "roofline": {"bound": "hbm", "kernel": "k_classify_bits", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": k1_bytes, "ms_per_launch": t_k1},
        "pipeline_roofline": {"achieved": pipe_gbs, "peak": peak, "unit": "GB/s",
                              "frac": pipe_gbs / peak, "algorithmic_bytes": alg_bytes,
                              "formula": "4P + 12V + 12T"},
        "stages_ms": {"classify": t_k1, "count_scan_incl_classify": t_count,
                      "generate": t_gen},
        "e2e": {"value": e2e_value, "unit": "cells/s", "h2d_bytes_per_step": 4 * P,
                "d2h_bytes_per_step": 12 * V + 12 * T, "ms_per_step": 1e3 * t_e2e,
                "steps": e2e_steps, "steps_in_flight": E,
                "h2d_field_copy_ms": h2d_ms, "h2d_link_gbs": h2d_gbs,
                "frac_of_h2d_floor": h2d_ms / (1e3 * t_e2e),
                "path": "C ABI; per step the field is copied from page-locked host memory to the "
                        "device (two halves on two streams) and the surface back to page-locked "
                        "host memory"},
        # per step: K1, K2a, K2b and K3 per slab, or (fused, one slab) the
        # fused classify + count, the scan and K3
        "gpu_launches": (3 if args.fused and slab_count == 1 else 4 * slab_count) * args.steps,
        "clocks": clocks,
    }
    if not args.no_extras:
        line.update(extra_measurements(field, grid, dims, iso, peak, stream, dev))
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the CPU-baseline leg: the reference on the whole field checks the
        # timed frames' surface bit for bit, its FP64 twin states the float32
        # error, and the bounded samples time the CPU implementation
        fh = field.cpu().numpy()
        line["parity"] = reference_parity(fh, dims, spacing, iso, verts_pipe, conn_pipe)
        line["fp64_error"] = fp64_error_statement(fh, dims, spacing, iso, grid, field, verts_pipe,
                                                  conn_pipe, scratch)
        cb = cpu_baseline(fh, dims, spacing, iso, args.cpu_seconds)
        line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
        cs = cpu_baseline(fh, dims, spacing, iso, args.cpu_seconds, threads=1)
        line["cpu_baseline_serial"] = {k: cs[k] for k in ("value", "unit", "cores", "kind",
                                                          "sample")}
        line["cpu_baseline_serial"]["adapter"] = (
            "Serial: one thread, the std:: algorithms of DeviceAdapterAlgorithmSerial.h")
        if "slice" in line:
            sl = cpu_slice_baseline(dims, spacing, (0.45, 0.5, 0.55), (0.3, 0.9, -0.3), 4.0)
            sl["gpu_over_cpu"] = line["slice"]["cells_per_s"] / sl["value"]
            line["slice"]["cpu_baseline"] = sl
        if "reference_mc_benchmark" in line:
            rb = cpu_reference_benchmark(128)
            gb = line["reference_mc_benchmark"]["dim128"]
            rb["gpu_over_cpu"] = {k: gb[k]["cells_per_s"] / rb[k] for k in ("plain", "remove_duplicates")}
            line["reference_mc_benchmark"]["cpu_baseline"] = rb
        if "mandelbulb" in line:
            mb = cpu_mandelbulb_baseline(200, 3.0)
            mb["gpu_over_cpu"] = line["mandelbulb"]["n200"]["points_per_s"] / mb["value"]
            line["mandelbulb"]["cpu_baseline"] = mb
        if "marching_tetrahedra" in line:
            import torch
            from daxtoolkit_gb300 import synthetic
            mt = line["marching_tetrahedra"]
            n = mt["n"]
            fm = synthetic.blob_field((n, n, n), 8, seed=0).numpy().ravel()
            cm = cpu_mt_baseline((n, n, n), (1.0 / (n - 1),) * 3, fm, 0.5, 4.0)
            cm["gpu_over_cpu"] = mt["tetrahedra_per_s_merged"] / cm["value"]
            mt["cpu_baseline"] = cm
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
