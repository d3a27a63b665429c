"""Benchmark of the fused LBM step (MLUPS and fraction of the HBM roofline).

Default workload: lid-driven cavity, D3Q19, recursive-regularised collision, FP32
populations, 256^3 cells (the size the roofline target is stated at), lattice units
nu = 0.032, lid u = 0.05; synthetic data (the reference publishes no data set).
A "step" is one LBM time step over the whole lattice (k_bulk + k_special).

value  : device-resident throughput, MLUPS = cells * steps / time (CUDA events on the
         library's stream, max over ranks).
e2e    : the same metric through the C ABI with host buffers: every e2e step uploads the
         populations from pinned host memory, runs E2E_INNER time steps and downloads the
         populations, MLUPS counted over the inner steps; per_output_interval: OUTPUT_INTERVAL
         steps and one download, the reference driver's output cadence on its cavity case.
roofline: k_bulk, algorithmic bytes = 152 B (D3Q19 FP32) per updated cell, divided by its
         average launch time from CUDA events; peak = measured HBM copy bandwidth.
variants: the FP16-shifted storage and the D3Q27 lattice on the same grid, and the
         1024x256x4 cylinder-channel configuration, measured the same way.

Multi-GPU: the step does not shard (one lattice per GPU, no halo exchange); under torchrun
each rank runs an independent replica (weak scaling) and rank 0 reports the aggregate.

--impl reference: the reference's own k_streamingCollision compiled as C (oracle/_ref) on
all host cores, same workload and metric.
"""
from __future__ import annotations

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

BYTES_PER_CELL = {(19, "fp32"): 152, (19, "fp16s"): 76, (19, "bf16s"): 76, (27, "fp32"): 216, (27, "fp16s"): 108,
                  (27, "bf16s"): 108}
E2E_INNER = 100
# the reference's own output cadence for its lid-driven cavity case (testCases/cavityFlow/input.txt:
# outInterval 1000): each output downloads the populations once (write.hpp)
OUTPUT_INTERVAL = 1000


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[4 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def make_workload(name):
    from lbffs_gb300 import case as K
    from lbffs_gb300 import geometry as G
    if name == "cavity256":
        n = 256
        c = K.make_case(n, n, n, 19, K.cavity_faces(0.05), nu=0.032)
        return c, dict(collision="rr", sgs="smag", wall="bb", les=0.0)
    if name == "cavity128":
        n = 128
        c = K.make_case(n, n, n, 19, K.cavity_faces(0.05), nu=0.032)
        return c, dict(collision="rr", sgs="smag", wall="bb", les=0.0)
    if name == "cavity256x64":
        c = K.make_case(256, 256, 64, 19, K.cavity_faces(0.05), nu=0.032)
        return c, dict(collision="rr", sgs="smag", wall="bb", les=0.0)
    if name == "cavity128_q27":
        n = 128
        c = K.make_case(n, n, n, 27, K.cavity_faces(0.05), nu=0.032)
        return c, dict(collision="rr", sgs="smag", wall="ibb", les=0.0)
    if name == "cavity256x64_q27":
        c = K.make_case(256, 256, 64, 27, K.cavity_faces(0.05), nu=0.032)
        return c, dict(collision="rr", sgs="smag", wall="ibb", les=0.0)
    if name == "cavity256_q27":
        n = 256
        c = K.make_case(n, n, n, 27, K.cavity_faces(0.05), nu=0.032)
        return c, dict(collision="rr", sgs="smag", wall="ibb", les=0.0)
    if name == "cylinder1024":
        rng = np.random.default_rng(1)
        cy = 128 + rng.uniform(-0.5, 0.5)
        solid, sdf = G.cylinder_z(1024, 256, 4, 256.0, cy, 20.0)
        c = K.make_case(1024, 256, 4, 19, K.channel_faces(0.05), nu=0.02, solid=solid, sdf=sdf)
        return c, dict(collision="rr", sgs="smag", wall="ibb", les=0.0)
    if name == "step768_q27":
        # backward-facing step: 768x192x192, step 64 high ending at x = 128, inlet 0.06 with a
        # seeded +-1 % per-cell perturbation, Re 5500 on the step height, Smagorinsky LES (Cs 0.1) with
        # Van Driest wall damping, sponge over the last 64 cells before the Geier outlet
        nx, ny, nz, h = 768, 192, 192, 64
        solid, sdf = G.backward_step(nx, ny, nz, 128, h)
        c = K.make_case(nx, ny, nz, 27, K.channel_faces(0.06, top_bottom=K.BOUNCEBACK, z_periodic=True),
                        nu=0.06 * h / 5500.0, solid=solid, sdf=sdf)
        rng = np.random.default_rng(3)
        inlet = c.boundary1 == K.FIXEDVELOCITY
        c.u0[inlet] *= (1.0 + rng.uniform(-0.01, 0.01, int(inlet.sum()))).astype(np.float32)
        c.f = None
        return c, dict(collision="rr", sgs="smag", wall="ibb", les=1.0, spz=64.0 / nx, rest=True, damping="vandriest")
    if name == "step384_q27":
        # the backward-facing step at half size in each direction (profiling size, populations larger
        # than L2): the same boundaries, LES, damping and sponge as the 768x192x192 case
        nx, ny, nz, h = 384, 96, 96, 32
        solid, sdf = G.backward_step(nx, ny, nz, 64, h)
        c = K.make_case(nx, ny, nz, 27, K.channel_faces(0.06, top_bottom=K.BOUNCEBACK, z_periodic=True),
                        nu=0.06 * h / 5500.0, solid=solid, sdf=sdf)
        c.f = None
        return c, dict(collision="rr", sgs="smag", wall="ibb", les=1.0, spz=32.0 / nx, rest=True, damping="vandriest")
    if name == "bluff1024_q27":
        # bluff body from a seeded procedural STL: a closed ellipsoid mesh of 20,000 triangles with
        # 5 % radial noise, 400 cells long, in a 1024x384x384 D3Q27 channel (inlet 0.05, Geier outlet,
        # free-slip y faces, periodic z), nu 1e-5, LES Cs 0.1, IBB on the STL links; voxelised and
        # given its wall distance on the device.  Upstream IBM cylinder: D = 32, 512 markers (16
        # rings of 32), sinusoidal y motion of amplitude 16 cells and period 4000 steps.
        nx, ny, nz = 1024, 384, 384
        nu = 1e-5
        faces = K.channel_faces(0.05)
        boundary, b1, b2, b3, u0, v0, w0 = K.face_arrays(nx, ny, nz, faces)
        omega = np.full(nx * ny * nz, K.omega_from_nu(nu), np.float32)
        c = K.Case(nx, ny, nz, 27, dict(faces), boundary, b1, b2, b3, u0, v0, w0, None, None, None, omega, None, nu)
        tris = G.ellipsoid_mesh(2025, 51, 200, (560.0, 192.0, 192.0), (200.0, 60.0, 60.0), noise=0.05)
        markers = np.concatenate([G.cylinder_markers(32, 160.0, 192.0, 184.0 + z, 16.0) for z in range(16)])
        return c, dict(collision="rr", sgs="smag", wall="ibb", les=1.0, rest=True,
                       stl=(tris.astype(np.float32), G.facet_normals(tris).astype(np.float32)), markers=markers,
                       motion=dict(amp=(0.0, 16.0, 0.0), period=4000.0))
    raise KeyError(name)


def serving_requests(n, step_scale, seed=2024):
    """The serving workload: Poisson arrivals (mean 200/s), each a lid-driven cavity or a channel
    with a cylinder (50/50), grid edge log-uniform in [24, 192] cells, Re uniform in [50, 400],
    FP32 or FP16-shifted storage (50/50), uniform in [2000, 20000] steps times step_scale."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    for _ in range(n):
        t += rng.exponential(1.0 / 200.0)
        out.append(dict(t=t, kind="cavity" if rng.random() < 0.5 else "channel",
                        edge=int(round(float(np.exp(rng.uniform(np.log(24.0), np.log(192.0)))))),
                        re=float(rng.uniform(50.0, 400.0)), storage="fp32" if rng.random() < 0.5 else "fp16s",
                        steps=max(1, int(round(float(rng.uniform(2000, 20000)) * step_scale))),
                        jitter=float(rng.uniform(-0.5, 0.5))))
    return out


def serving_case(r):
    """Arrays of one request (populations start from rest on the device)."""
    from lbffs_gb300 import case as K
    from lbffs_gb300 import geometry as G
    n = r["edge"]
    if r["kind"] == "cavity":
        c = K.make_case(n, n, n, 19, K.cavity_faces(0.05), nu=0.05 * n / r["re"])
        wall = "bb"
    else:  # 2n x n x n/4 channel, cylinder of diameter n/5 a quarter length downstream, Re on D
        nx, ny, nz = 2 * n, n, max(4, n // 4)
        d = n / 5.0
        solid, sdf = G.cylinder_z(nx, ny, nz, nx / 4.0, ny / 2.0 + r["jitter"], d / 2.0)
        c = K.make_case(nx, ny, nz, 19, K.channel_faces(0.05), nu=0.05 * d / r["re"], solid=solid, sdf=sdf)
        wall = "ibb"
    c.f = None
    return c, wall


def _serial(reqs, cases, device, per_step_sync):
    """Each request alone on a fresh Lattice, in arrival order.  per_step_sync: one time step per
    call followed by a synchronize, as the reference driver runs k_streamingCollision and
    queue.finish() every step (ns.cpp:514-603); otherwise all steps in one asynchronous call."""
    import lbffs_gb300 as L
    t0 = time.perf_counter()
    lat_ms, keep = [], {}
    for k, (r, (c, wall)) in enumerate(zip(reqs, cases)):
        wait = t0 + r["t"] - time.perf_counter()
        if wait > 0:
            time.sleep(wait)
        lat = L.Lattice(c.nx, c.ny, c.nz, storage=r["storage"], wall=wall, device=device)
        for name in ("boundary", "boundary1", "boundary2", "boundary3", "u0", "v0", "w0", "solid", "nei_solid", "sdf",
                     "omega"):
            lat.upload(name, getattr(c, name))
        lat.init_rest()
        if per_step_sync:
            for s in range(r["steps"]):
                lat.step(1, store_fields=1 if s == r["steps"] - 1 else 0)
                lat.synchronize()
        else:
            lat.step(r["steps"], store_fields=1)
            lat.synchronize()
        u = lat.download("u")
        if k % 8 == 0:
            keep[k] = u
        lat.close()
        lat_ms.append(time.perf_counter() - (t0 + r["t"]))
    return time.perf_counter() - t0, lat_ms, keep


def run_serving(n_req, step_scale, device, budget_gb=150.0, serial=True):
    """Served (continuous batching) vs serial plain launches of the same requests and arrivals
    (serial=False: the served run alone)."""
    from lbffs_gb300.serve import Server
    reqs = serving_requests(n_req, step_scale)
    cases = [serving_case(r) for r in reqs]
    cells = [c.nx * c.ny * c.nz * r["steps"] for r, (c, _) in zip(reqs, cases)]
    bpc = [BYTES_PER_CELL[(19, r["storage"])] for r in reqs]

    if serial:
        t_plain, lat_plain, keep = _serial(reqs, cases, device, True)
        t_async, lat_async, _ = _serial(reqs, cases, device, False)
    else:
        t_plain, lat_plain, keep, t_async = float("nan"), [float("nan")], {}, float("nan")

    # served: the same arrivals, submitted from a client thread
    srv = Server(hbm_budget=int(budget_gb * (1 << 30)), max_cases=256, steps_per_round=16, device=device)
    ids = [None] * n_req
    t0 = time.perf_counter()

    def client():
        for k, (r, (c, wall)) in enumerate(zip(reqs, cases)):
            wait = t0 + r["t"] - time.perf_counter()
            if wait > 0:
                time.sleep(wait)
            ids[k] = srv.submit(c, r["steps"], storage=r["storage"], wall=wall, from_rest=True)

    th = threading.Thread(target=client)
    th.start()
    th.join()
    for cid in ids:
        srv.wait(cid, 3600.0)
    t_served = time.perf_counter() - t0
    st = srv.stats()
    same = all(np.array_equal(srv.result(ids[k], "u"), u) for k, u in keep.items())
    srv.close()
    peak, _ = peaks()
    tot = float(sum(cells))
    bytes_tot = float(sum(cl * b for cl, b in zip(cells, bpc)))
    return {"requests": n_req, "step_scale": step_scale,
            "sample": f"{n_req} requests of the serving workload (seed 2024), steps scaled by {step_scale}",
            "solves_per_s": n_req / t_served, "serial_solves_per_s": n_req / t_plain,
            "speedup_vs_serial": t_plain / t_served,
            "serial_async_solves_per_s": n_req / t_async, "speedup_vs_serial_async": t_async / t_served,
            "latency_p50_s": st["latency_p50_s"], "latency_p99_s": st["latency_p99_s"],
            "queue_wait_p99_s": st["queue_wait_p99_s"],
            "serial_latency_p50_s": float(np.percentile(lat_plain, 50)),
            "serial_latency_p99_s": float(np.percentile(lat_plain, 99)),
            "MLUPS": tot / t_served / 1e6, "serial_MLUPS": tot / t_plain / 1e6,
            "hbm_frac": bytes_tot / t_served / 1e9 / peak,
            "hbm_peak_GB": st["hbm_peak"] / 1e9, "rounds": st["rounds"], "graph_builds": st["graph_builds"],
            "gpu_busy_s": st["gpu_busy_s"], "build_s": st["build_s"], "mean_resident": st["mean_resident"],
            "served_s": t_served,
            "identical_to_serial": bool(same) if serial else None, "compared": len(keep),
            "serial": "one Lattice per request in arrival order, one step per call + synchronize "
                      "(the reference driver's launch + queue.finish per step)"}


def describe(name, storage):
    return {"cavity256": f"lid-driven cavity D3Q19 RR {storage.upper()} 256^3, nu=0.032, lid 0.05 (synthetic)",
            "cavity128": f"lid-driven cavity D3Q19 RR {storage.upper()} 128^3 (synthetic, profiling size)",
            "cavity256x64": f"lid-driven cavity D3Q19 RR {storage.upper()} 256x256x64 (synthetic, profiling size: "
                            "the 256-cell rows of the 256^3 case, populations larger than L2)",
            "cavity256_q27": f"lid-driven cavity D3Q27 RR {storage.upper()} 256^3 (synthetic)",
            "cavity128_q27": f"lid-driven cavity D3Q27 RR {storage.upper()} 128^3 (synthetic, profiling size)",
            "cavity256x64_q27": f"lid-driven cavity D3Q27 RR {storage.upper()} 256x256x64 (synthetic, profiling size: "
                                "populations larger than L2)",
            "cylinder1024": f"cylinder channel D3Q19 RR IBB {storage.upper()} 1024x256x4, D=40, Re=100 (synthetic)",
            "step768_q27": f"backward-facing step D3Q27 RR IBB LES (Van Driest damping) {storage.upper()} 768x192x192, "
                           "step 64, Re 5500, "
                           "sponge 64 cells (synthetic)",
            "step384_q27": f"backward-facing step D3Q27 RR IBB LES {storage.upper()} 384x96x96, step 32 (synthetic, "
                           "profiling size)",
            "bluff1024_q27": f"bluff body D3Q27 RR IBB LES {storage.upper()} 1024x384x384, 20,000-triangle noisy "
                             "ellipsoid (400 cells) voxelised on the device, IBM cylinder D=32 with 512 markers "
                             "(synthetic)"}[name]


BULK_KIND = 0  # D3Q19 bulk kernel variant (--bulk-kind)
BORDER_PULLS = 1  # face streaming read where it lies (1) or from a ghost layer filled every step (0)


def run_device(name, storage, steps, warmup, device, timing_pass=True):
    import torch
    import lbffs_gb300 as L
    c, sel = make_workload(name)
    lat = L.Lattice(c.nx, c.ny, c.nz, q=c.q, storage=storage, collision=sel["collision"], sgs=sel["sgs"],
                    wall=sel["wall"], device=device, damping=sel.get("damping", "wall"))
    if c.q == 19:
        lat.set_bulk_kernel(BULK_KIND)
    lat.set_border_pulls(BORDER_PULLS)
    if sel.get("rest"):
        for name in ("boundary", "boundary1", "boundary2", "boundary3", "u0", "v0", "w0", "solid", "nei_solid", "sdf",
                     "omega"):
            if getattr(c, name) is not None:
                lat.upload(name, getattr(c, name))
        lat.init_rest()
    else:
        lat.load_case(c)
    setup = {}
    if sel.get("stl") is not None:
        # solid / neiSolid and the LES wall distance from the STL, on the device
        verts, normals = sel["stl"]
        t0 = time.perf_counter()
        lat.voxelize(verts)
        t1 = time.perf_counter()
        lat.build_sdf(verts, normals)
        t2 = time.perf_counter()
        setup = {"voxelize_s": t1 - t0, "sdf_s": t2 - t1, "triangles": int(verts.shape[0])}
    if sel.get("markers") is not None:
        lat.set_markers(sel["markers"])
        lat.set_motion(**sel.get("motion", {}))
    spz = sel.get("spz", 0.1)
    stream = torch.cuda.ExternalStream(lat.stream(), device=device)
    lat.step(warmup, les=sel["les"], spz_width=spz, store_fields=0)
    lat.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if torch.distributed.is_initialized():
        torch.distributed.barrier()
    torch.cuda.synchronize(device)
    e0.record(stream)
    lat.step(steps, les=sel["les"], spz_width=spz, store_fields=0)
    e1.record(stream)
    e1.synchronize()
    lat.synchronize()
    torch.cuda.synchronize(device)
    ms = e0.elapsed_time(e1)
    counts = lat.cell_counts()
    out = {"ms_per_step": ms / steps, "cells": c.elements, "fluid": counts["fluid"], "special": counts["special"],
           # k_bulk every step, k_special when the case has special cells, the ghost fill when the step
           # does not pull across the border itself (refined by the timing pass's launch counts)
           "launches_per_step": (3 if counts["special"] > 0 else 2) + (4 if sel.get("markers") is not None else 0),
           "lat": lat, "case": c, "sel": sel, "setup": setup}
    if timing_pass:
        lat.set_timing(True)
        lat.step(steps, les=sel["les"], spz_width=spz, store_fields=0)
        bulk_ms, n = lat.kernel_time("bulk")
        sp_ms, nsp = lat.kernel_time("special")
        h_ms, nh = lat.kernel_time("halo")
        i_ms, ni = lat.kernel_time("ibm")
        lat.set_timing(False)
        out["ibm_ms"] = i_ms / max(ni, 1)
        # launches of the library's kernels per step: bulk, boundary, ghost fill (none when the step pulls
        # across the border itself), IBM sub-step (four kernels)
        out["launches_per_step"] = (n + nsp + nh + 4 * ni) / steps
        out["bulk_ms"] = bulk_ms / max(n, 1)
        out["special_ms"] = sp_ms / max(nsp, 1)
        out["halo_ms"] = h_ms / max(nh, 1)
    return out


def force_series(res, samples=20, every=250):
    """Drag / lift coefficients of the cylinder channel over time from the FP64 wall-force sum
    (lbffs_force_sum), normalised as D3Q19_opencl/write.hpp:104 in lattice units: F / (1/2 rho_av U^2 D nz)
    with the inlet speed U = 0.05, the diameter D = 40 cells and the z extent nz (the frontal area)."""
    lat, c = res["lat"], res["case"]
    n_fluid = float((c.solid == 0).sum()) if c.solid is not None else float(c.elements)
    scale = 1.0 / (0.5 * 0.05 ** 2 * 40.0 * c.nz)
    out = []
    for s in range(samples):
        lat.step(every, store_fields=0)
        fw = lat.force_sum()
        rho_av = lat.mass() / n_fluid
        out.append([(s + 1) * every, fw[0] * scale / rho_av, fw[1] * scale / rho_av])
    return {"every_steps": every, "t_cx_cy": [[int(t), round(float(a), 6), round(float(b), 6)] for t, a, b in out],
            "note": "after the timed steps, from the channel started at rest (start-up transient)"}


def _cpulist(text):
    out = set()
    for part in text.strip().split(","):
        if part:
            a, _, b = part.partition("-")
            out.update(range(int(a), int(b or a) + 1))
    return out


def gpu_local_cpus(device):
    """(NUMA node, host CPUs of that node this process may run on) of the GPU's PCI device, or
    (None, None) when the system does not say."""
    import torch
    try:
        p = torch.cuda.get_device_properties(device)
        bus = f"{p.pci_domain_id:04x}:{p.pci_bus_id:02x}:{p.pci_device_id:02x}.0"
        node = int(open(f"/sys/bus/pci/devices/{bus}/numa_node").read())
        if node < 0:
            return None, None
        cpus = _cpulist(open(f"/sys/devices/system/node/node{node}/cpulist").read()) & os.sched_getaffinity(0)
        return (node, cpus) if cpus else (None, None)
    except Exception:
        return None, None


def run_e2e(res, steps, device):
    """Upload from pinned host memory, E2E_INNER steps, download: timed with CUDA events, the copies inside.
    The pinned buffers are allocated from a CPU of the GPU's own NUMA node when the system names one,
    so that their pages lie in the memory next to the GPU."""
    import torch
    lat, c, sel = res["lat"], res["case"], res["sel"]
    f0 = c.f
    if f0 is None:  # a case started from rest on the device: its host populations are the weights
        from lbffs_gb300 import case as K
        f0 = np.repeat(K.lattice(c.q)[1], c.elements)
    node, cpus = gpu_local_cpus(device)
    keep_aff = os.sched_getaffinity(0)
    if cpus:
        os.sched_setaffinity(0, cpus)
    try:
        host_in = torch.from_numpy(f0).pin_memory()
        host_out = torch.empty_like(host_in).pin_memory()
        host_out.zero_()  # pages placed by this thread
    finally:
        os.sched_setaffinity(0, keep_aff)
    stream = torch.cuda.ExternalStream(lat.stream(), device=device)
    import ctypes as C
    lib = lat.lib

    def one(inner=E2E_INNER, upload=True):
        if upload:
            rc = lib.lbffs_upload(lat.h, 0, C.c_void_p(host_in.data_ptr()), host_in.numel() * 4)
            assert rc == 0, lib.lbffs_last_error(lat.h)
        lat.step(inner, les=sel["les"], store_fields=0)
        rc = lib.lbffs_download(lat.h, 0, C.c_void_p(host_out.data_ptr()), host_out.numel() * 4)
        assert rc == 0, lib.lbffs_last_error(lat.h)

    one()
    n_e2e = max(1, min(steps, 3))
    torch.cuda.synchronize(device)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record(stream)
    for _ in range(n_e2e):
        one()
    e1.record(stream)
    e1.synchronize()
    wall = time.perf_counter() - t0
    ms = max(e0.elapsed_time(e1), wall * 1e3)
    mlups = c.elements * E2E_INNER * n_e2e / (ms * 1e-3) / 1e6
    # the reference driver's cadence: OUTPUT_INTERVAL steps, then the populations downloaded
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    e0.record(stream)
    one(OUTPUT_INTERVAL, upload=False)
    e1.record(stream)
    e1.synchronize()
    ms_out = max(e0.elapsed_time(e1), (time.perf_counter() - t0) * 1e3)
    return {"value": mlups, "unit": "MLUPS", "h2d_bytes_per_step": int(host_in.numel() * 4),
            "d2h_bytes_per_step": int(host_out.numel() * 4), "inner_steps": E2E_INNER, "e2e_steps": n_e2e,
            "ms_per_e2e_step": ms / n_e2e, "host_numa_node": node,
            "cadence": f"each e2e step: upload of all populations, {E2E_INNER} time steps, download of all "
                       "populations",
            "per_output_interval": {"steps": OUTPUT_INTERVAL, "d2h_bytes": int(host_out.numel() * 4),
                                    "value": c.elements * OUTPUT_INTERVAL / (ms_out * 1e-3) / 1e6,
                                    "unit": "MLUPS",
                                    "cadence": f"{OUTPUT_INTERVAL} time steps, then one download of all "
                                               "populations (the reference cavity case's outInterval)"}}


def cpu_reference_mlups(nx, ny, nz, steps, threads=0, kind_pref="reference"):
    """The reference kernel compiled as C (oracle/_ref) or the CPU oracle, all host threads."""
    from lbffs_gb300 import case as K
    from oracle import ref as R
    c = K.make_case(nx, ny, nz, 19, K.cavity_faces(0.05), nu=0.032)
    kind = "reference" if (kind_pref == "reference" and R.available(19, "smag", "bb", "f32")) else "port"
    solver = R.RefSolver(c, real="f32", nthreads=threads) if kind == "reference" else \
        R.OracleSolver(c, real="f32", nthreads=threads)
    solver.step(1)
    t0 = time.perf_counter()
    solver.step(steps)
    dt = time.perf_counter() - t0
    return c.elements * steps / dt / 1e6, kind, (threads or os.cpu_count())


def traffic_from_profile():
    """Per-launch DRAM bytes of k_bulk from the committed ncu summary, if present."""
    p = os.path.join(ROOT, "profiles", "k_bulk_d3q19_fp32_cavity.md")
    try:
        for line in open(p):
            if line.startswith("traffic_bytes_per_launch_256:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cavity256")
    ap.add_argument("--storage", default="fp32")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--requests", type=int, default=512, help="serving workload: number of requests")
    ap.add_argument("--step-scale", type=float, default=1.0, help="serving workload: step count scale")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-serial", action="store_true",
                    help="serving workload: the served run alone, without the serial baselines")
    ap.add_argument("--bulk-kind", type=int, default=0, choices=[0, 1],
                    help="D3Q19 bulk kernel: 0 per-thread loads, 1 row-staged bulk copies")
    ap.add_argument("--border-pulls", type=int, default=1, choices=[0, 1],
                    help="1: populations crossing the grid's border read where the face streaming takes "
                         "them (where the faces allow); 0: from a ghost layer filled before every step")
    ap.add_argument("--profile", action="store_true",
                    help="device-timed steps only (no e2e, CPU baseline or variants): the command ncu captures")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    global BULK_KIND, BORDER_PULLS
    BULK_KIND = args.bulk_kind
    BORDER_PULLS = args.border_pulls

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return 0
        from oracle.build import build_oracle
        build_oracle()
        n = 256
        # all host threads, the full workload; each step is one reference NDRange launch over 256^3 cells
        from lbffs_gb300 import case as K
        from oracle import ref as R
        c = K.make_case(n, n, n, 19, K.cavity_faces(0.05), nu=0.032)
        kind = "reference" if R.available(19, "smag", "bb", "f32") else "port"
        solver = R.RefSolver(c, real="f32") if kind == "reference" else R.OracleSolver(c, real="f32")
        solver.step(args.warmup)
        t0 = time.perf_counter()
        solver.step(args.steps)
        dt = time.perf_counter() - t0
        mlups = c.elements * args.steps / dt / 1e6
        line = {"impl": "reference", "metric": "MLUPS", "value": mlups, "unit": "MLUPS", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": {"workload": describe("cavity256", "fp32"), "cells": c.elements},
                "cpu_baseline": {"value": mlups, "unit": "MLUPS", "cores": os.cpu_count(), "kind": kind,
                                 "sample": f"256^3 cavity, {args.steps} steps (the full workload)"},
                "e2e": {"value": mlups, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    import torch
    if world > 1:
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    device = local if world > 1 else 0
    torch.cuda.set_device(device)

    if args.workload == "serving":
        if rank == 0:
            out = run_serving(args.requests, args.step_scale, device, serial=not args.no_serial)
            out.update({"metric": "served solves/s", "unit": "solves/s", "value": out["solves_per_s"],
                        "higher_is_better": True, "n_gpus": 1, "dtype": "f32/fp16s", "data": "synthetic"})
            print(json.dumps(out))
        return 0
    if args.profile:
        res = run_device(args.workload, args.storage, args.steps, args.warmup, device, timing_pass=False)
        print(json.dumps({"workload": describe(args.workload, args.storage), "ms_per_step": res["ms_per_step"],
                          "MLUPS": res["cells"] / (res["ms_per_step"] * 1e-3) / 1e6}))
        return 0
    with ClockSampler(device) as clk:
        res = run_device(args.workload, args.storage, args.steps, args.warmup, device)
    clocks = clk.summary()
    ms = res["ms_per_step"]
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    mlups = world * res["cells"] / (ms * 1e-3) / 1e6
    e2e = run_e2e(res, args.steps, device)
    if world > 1:
        t = torch.tensor([e2e["value"]], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MIN)
        e2e["value"] = float(t.item()) * world

    q = res["case"].q
    bpc = BYTES_PER_CELL[(q, args.storage)]
    peak, peak_kind = peaks()
    n_bulk = res["fluid"] - res["special"]
    achieved = bpc * n_bulk / (res["bulk_ms"] * 1e-3) / 1e9
    traffic = traffic_from_profile() if (args.workload == "cavity256" and args.storage == "fp32") else None

    variants = {}
    if rank == 0 and not args.no_variants and args.workload == "cavity256":
        for vname, vst in (("cavity256", "fp16s"), ("cavity256", "bf16s"), ("cavity256_q27", "fp32"),
                           ("cavity256_q27", "fp16s"), ("cylinder1024", "fp32"), ("cylinder1024", "fp16s"),
                           ("step768_q27", "fp32"), ("step768_q27", "fp16s"), ("bluff1024_q27", "fp16s")):
            try:
                big = vname in ("step768_q27", "bluff1024_q27")
                r = run_device(vname, vst, min(args.steps, 50) if big else args.steps, args.warmup, device)
                vq = r["case"].q
                vb = BYTES_PER_CELL[(vq, vst)]
                vn = r["fluid"] - r["special"]
                variants[f"{vname}_{vst}"] = {
                    "workload": describe(vname, vst), "MLUPS": r["cells"] / (r["ms_per_step"] * 1e-3) / 1e6,
                    "ms_per_step": r["ms_per_step"], "bulk_ms": r["bulk_ms"], "special_ms": r["special_ms"],
                    "halo_ms": r["halo_ms"],
                    "bulk_GBps": vb * vn / (r["bulk_ms"] * 1e-3) / 1e9,
                    "bulk_frac_of_peak": vb * vn / (r["bulk_ms"] * 1e-3) / 1e9 / peak,
                    "bytes_per_cell": vb}
                if vst == "bf16s":
                    variants[f"{vname}_{vst}"]["accuracy"] = (
                        "below the 1e-3 velocity-error bar of reduced-precision storage (FP16S meets it); "
                        "not an equal alternative to FP16S")
                if vname == "cylinder1024":
                    variants[f"{vname}_{vst}"]["force_coefficients"] = force_series(r)
                if r["setup"]:
                    variants[f"{vname}_{vst}"]["setup"] = r["setup"]
                    variants[f"{vname}_{vst}"]["ibm_ms"] = r.get("ibm_ms")
                    variants[f"{vname}_{vst}"]["wall_force"] = [float(x) for x in r["lat"].force_sum()]
                r["lat"].close()
                del r
            except Exception as ex:  # a failing variant must not hide the headline
                variants[f"{vname}_{vst}"] = {"error": str(ex)[:200]}

    serving = None
    if rank == 0 and not args.no_serving and args.workload == "cavity256":
        try:
            serving = run_serving(48, 0.1, device)
        except Exception as ex:  # the serving sample must not hide the headline
            serving = {"error": str(ex)[:300]}

    cpu = None
    if rank == 0:
        try:
            cm, kind, cores = cpu_reference_mlups(128, 128, 128, 60)
            cpu = {"value": cm, "unit": "MLUPS", "cores": cores, "kind": kind,
                   "sample": "128^3 lid-driven cavity D3Q19 FP32, 60 steps, all host threads"}
        except Exception as ex:
            cpu = {"value": None, "unit": "MLUPS", "cores": os.cpu_count(), "kind": "reference",
                   "sample": f"unavailable: {str(ex)[:120]}"}

    if rank == 0:
        line = {
            "metric": "MLUPS", "value": mlups, "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if args.storage == "fp32" else f"f32 compute, {args.storage} storage",
            "data": "synthetic",
            "config": {"workload": describe(args.workload, args.storage), "cells": res["cells"],
                       "lattice": f"D3Q{q}", "storage": args.storage, "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (populations %.2f GB per copy)" % (q * res["cells"] * bpc / 2 / q / 1e9)},
            "e2e": e2e,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "kernel": "k_bulk", "bytes_per_cell": bpc, "cells_per_launch": n_bulk,
                         "launch_ms": res["bulk_ms"], "peak_source": f"{peak_kind} hbm_gbs",
                         "step_kernels_ms": {"k_bulk": res["bulk_ms"], "k_special": res["special_ms"],
                                             "k_halo": res["halo_ms"]}},
            "cpu_baseline": cpu,
            "clocks": clocks,
            "gpu_launches": int(round(res["launches_per_step"] * args.steps)),
            "variants": variants,
            "serving": serving,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
