#!/usr/bin/env python
"""Benchmark of the symmetry-reduced Hamiltonian application (mul! on a ReducedOperatorRepresentation).

Metric: reduced H*x throughput in GB/s of the byte model below, as a fraction of the measured HBM
peak, plus the time to E0 by Lanczos in FP64 and in mixed precision.

A step is one H*x over the whole sector.  Default workload: spin-1/2 Heisenberg chain L=24, periodic,
J=1, 2Sz=0, momentum 0 (112,720 representatives), mixed precision (complex64 vectors, FP32
accumulation).  Inputs are seeded complex Gaussian vectors generated on the GPU; successive steps
cycle through a pool of input/output vectors larger than twice the L2 cache, so each step reads its
x from HBM.  The operator tables (representatives, terms) stay resident.

Byte model per H*x (s_c = 8 for complex64, 16 for complex128):
    B = N_r * (8 + 8 + 2 s_c) + NNZ_off * (s_c + 8)
N_r rows (representative word + orbit norm + x_r + y_r) and NNZ_off off-diagonal elements whose target
lands on a representative (x gather + one table key).  NNZ_off is counted exactly on the GPU.  With a
parent-state map (default when it fits; --no-map to canonicalise instead) a target costs one 4- or
8-byte map entry instead of the key read; the model is kept as the fixed measure of work.

Arms:
  (default)         the GPU path (libedgpu.so) -- device-resident `value`, host-buffer `e2e` through the
                    C ABI (edgpu_mul with complex128 host vectors, copies inside the timed region).
  --impl reference  the CPU restatement of the reference's mul! (binary search over the parent basis,
                    parent-sized mapping tables, rows split statically over all host threads), FP64,
                    each step a block of rows of the same workload.
Multi-GPU (torchrun): replicas -- every rank applies the same workload on its own GPU; value sums the
ranks' bytes over the slowest rank's time.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(ROOT, "exactdiagonalization.jl_gb300")
for p in (PKG_DIR, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "reduced H*x GB/s & % of HBM peak; E0 time mixed vs FP64 at |dE|<1e-9"
L2_BYTES = 129 * 1024 * 1024
FALLBACK_HBM_GBS = 6800.0

WORKLOADS = {
    "chain24_k0": dict(kind="chain", L=24, k=0, jxy=1.0, jz=1.0, seed=2, lanczos_steps=200, reorth=True,
                       N_r=112720, nnz_off=1411488, steps=2000,
                       desc="spin-1/2 Heisenberg chain L=24 PBC J=1, 2Sz=0, momentum 0 (24-site translations)"),
    "chain16_full": dict(kind="chain_full", L=16, jxy=1.0, jz=1.0, seed=1, lanczos_steps=100, reorth=True,
                         N_r=12870, nnz_off=109824, steps=2000,
                         desc="spin-1/2 Heisenberg chain L=16 PBC J=1, 2Sz=0, no symmetry reduction"),
    "chain28_grad": dict(kind="chain_grad", L=28, k=0, seed=4, x_seed=5, gy_seed=6, cpu_feasible=True,
                         N_r=1432860, nnz_off=20803084, steps=200,
                         desc="spin-1/2 Heisenberg chain L=28 PBC, per-bond J_b = 0.5 + U[0,1) (seed 4), 2Sz=0, "
                              "momentum 0: forward H x, coupling gradient dL/dJ_b = Re<gy|H_b x>, adjoint H^dagger gy"),
    "chain28_k0": dict(kind="chain", L=28, k=0, jxy=1.0, jz=1.0, seed=5, lanczos_steps=200, reorth=True,
                       N_r=1432860, nnz_off=20803084, steps=500,
                       desc="spin-1/2 Heisenberg chain L=28 PBC, 2Sz=0, momentum 0"),
    "chain32_k0": dict(kind="chain", L=32, k=0, jxy=1.0, jz=1.0, seed=6, lanczos_steps=200, reorth=False,
                       cpu_feasible=False, N_r=18784170, nnz_off=None, steps=50,
                       desc="spin-1/2 Heisenberg chain L=32 PBC, 2Sz=0, momentum 0 (the smallest chain sector "
                            "whose x exceeds L2: the small case for profiling the slab product)"),
    "triangular6x5_allk": dict(kind="torus_allk", shape=(6, 5), nn=[(1, 0), (1, 1), (0, 1)],
                               nnn=[(2, 1), (1, 2), (-1, 1)], j1=1.0, j2=0.125, aniso=0.8, seed=3,
                               cpu_feasible=False, N_r=155117520, nnz_off=14441957888, steps=20,
                               desc="spin-1/2 XXZ J1-J2 triangular 6x5 torus (Jz/Jxy=0.8, J2/J1=0.125), 2Sz=0, "
                                    "all 30 momentum sectors in one batched persistent launch"),
    "triangular6x5_k1": dict(kind="torus", shape=(6, 5), k=(1, 0), nn=[(1, 0), (1, 1), (0, 1)],
                             nnn=[(2, 1), (1, 2), (-1, 1)], j1=1.0, j2=0.125, aniso=0.8, seed=3, lanczos_steps=200,
                             reorth=True, cpu_feasible=False, N_r=5170578, nnz_off=481397728, steps=200,
                             desc="spin-1/2 XXZ J1-J2 triangular 6x5 torus (Jz/Jxy=0.8, J2/J1=0.125), 2Sz=0, "
                                  "momentum (1,0) (one sector of the batched workload)"),
    "square6x6_c4v": dict(kind="torus_pg", shape=(6, 6), k=(0, 0), irrep="A1", nn=[(1, 0), (0, 1)],
                          nnn=[(1, 1), (1, -1)], j1=1.0, j2=0.5, aniso=1.0, seed=7, lanczos_steps=300, reorth=False,
                          cpu_feasible=False, N_r=31566122, nnz_off=2337741028, no_map=True, steps=50,
                          desc="spin-1/2 J1-J2 Heisenberg 6x6 torus (J2/J1=0.5), 2Sz=0, A1 at k=(0,0) of the "
                               "space group translations x C4v (288 elements; the general permutation path)"),
    "square6x6_k0": dict(kind="torus", shape=(6, 6), k=(0, 0), nn=[(1, 0), (0, 1)], nnn=[(1, 1), (1, -1)],
                         j1=1.0, j2=0.5, aniso=1.0, seed=7, lanczos_steps=300, reorth=False, cpu_feasible=False,
                         N_r=252091362, nnz_off=18669175824, steps=20,
                         desc="spin-1/2 J1-J2 Heisenberg 6x6 torus (J2/J1=0.5), 2Sz=0, momentum (0,0)"),
}


# ---------------------------------------------------------------------------------------------------
def bytes_model(n_rows: int, nnz_off: int, s_c: int) -> int:
    return n_rows * (8 + 8 + 2 * s_c) + nnz_off * (s_c + 8)


def hamiltonian_spec(wl):
    """(n_sites, bonds, jxy, jz, group shape, momentum) of a workload."""
    if wl["kind"] in ("chain", "chain_full"):
        L = wl["L"]
        bonds = [(i, (i + 1) % L) for i in range(L)]
        return L, bonds, [wl["jxy"]] * L, [wl["jz"]] * L, (L, 1), (wl.get("k", 0), 0)
    L1, L2 = wl["shape"]
    bonds, jxy, jz = [], [], []
    for vecs, j in ((wl["nn"], wl["j1"]), (wl["nnn"], wl["j2"])):
        for dx, dy in vecs:
            for y in range(L2):
                for x in range(L1):
                    bonds.append((x + L1 * y, (x + dx) % L1 + L1 * ((y + dy) % L2)))
                    jxy.append(j)
                    jz.append(j * wl["aniso"])
    return L1 * L2, bonds, jxy, jz, (L1, L2), wl.get("k", (0, 0))


def build_gpu_sectors(wl):
    """Every momentum sector of a torus workload: (spaces, operators, momenta, setup seconds)."""
    import edgpu
    from edgpu import lattice
    n, bonds, jxy, jz, shape, _ = hamiltonian_spec(wl)
    hs, _ = edgpu.spin_half_system(n)
    H = lattice.xxz_hamiltonian(hs, bonds, jxy, jz)
    t0 = time.perf_counter()
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0), lazy=True)
    momenta = [(m1, m2) for m2 in range(shape[1]) for m1 in range(shape[0])]
    spaces = [edgpu.symmetry_reduce(hsr, edgpu.translation_symops(shape, k)) for k in momenta]
    t_space = time.perf_counter() - t0
    oprs = [edgpu.represent(sp, H) for sp in spaces]
    return spaces, oprs, momenta, t_space


def build_maps(spaces, args):
    """Parent-state maps of reduced spaces (unless --no-map): {"entries", "bytes", "build_s"} or None."""
    import torch
    if args.no_map or not hasattr(spaces[0], "build_map"):
        return None
    if getattr(args, "workload_no_map", False):
        # the general permutation path canonicalises every parent state to build a map: the target
        # table is built from the representatives instead
        return {"built": False, "skipped": "large general group"}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    entries = nbytes = 0
    for sp in spaces:
        if not (sp.build_map(args.map_bytes) if args.map_bytes else sp.build_map()):
            return {"built": False}
        n, b = sp.map_info
        entries += n
        nbytes += n * b
    torch.cuda.synchronize()
    return {"built": True, "entries": entries, "bytes": nbytes, "build_s": time.perf_counter() - t0}


def build_tables(oprs, spaces, args):
    """Target tables of the pair-flip schedule (unless --no-table): {"built", "entries", "bytes",
    "build_s", "maps_freed"} or None.  Each table may take up to 80% of the free device memory; once
    every operator has one, the parent-state maps (used only to build them faster) are freed."""
    import torch
    if args.no_table or args.no_pair or not hasattr(oprs[0], "build_targets"):
        return None
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    entries = nbytes = 0
    for o in oprs:
        free, _ = torch.cuda.mem_get_info()
        if not o.build_targets(int(0.8 * free)):
            return {"built": False}
        n, b = o.targets_info
        entries += n
        nbytes += n * b
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    freed = False
    for sp in spaces:
        if hasattr(sp, "free_map") and sp.map_info[0] > 0:
            sp.free_map()
            freed = True
    return {"built": True, "entries": entries, "bytes": nbytes, "build_s": dt, "maps_freed": freed}


def build_slabs(opr, N, args):
    """Column-slab table of the operator (the autotuner times it against the one-pass schedules), unless
    --slab-mb 0; --slab-scaling picks its layout:
    {"built", "passes", "columns_per_slab", "entries", "bytes", "build_s", "scaled"} or None."""
    import torch
    if args.slab_mb <= 0 or not hasattr(opr, "build_slabs"):
        return None
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    free, _ = torch.cuda.mem_get_info()
    opr.slab_scaling(args.slab_scaling)
    built = opr.build_slabs(slab_bytes=int(args.slab_mb * (1 << 20)), max_bytes=int(0.8 * free))
    dt = time.perf_counter() - t0
    if not built:
        return {"built": False}
    passes, wc, entries = opr.slabs_info
    scaled = opr.slab_scaling()
    return {"built": True, "passes": passes, "columns_per_slab": wc, "entries": entries,
            "bytes": entries * 4 + passes * N + passes * ((N + 31) // 32) * 4 + (17 * N if scaled else 0),
            "build_s": dt, "scaled": scaled}


def build_gpu_operator(wl):
    import edgpu
    from edgpu import lattice
    n, bonds, jxy, jz, shape, k = hamiltonian_spec(wl)
    hs, _ = edgpu.spin_half_system(n)
    t0 = time.perf_counter()
    if wl["kind"] == "chain_full":
        space = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0))
    elif wl["kind"] == "torus_pg":
        hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0), lazy=True)
        space = edgpu.symmetry_reduce(hsr, lattice.square_c4v_symops(shape[0], k, wl["irrep"]))
    else:
        hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0), lazy=True)
        space = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(shape, k))
    t_space = time.perf_counter() - t0
    H = lattice.xxz_hamiltonian(hs, bonds, jxy, jz)
    opr = edgpu.represent(space, H)
    return space, opr, t_space


# ---------------------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms in the background."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.samples = []
        self.proc = None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", str(device_index)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.time(), [v.strip() for v in line.split(",")]))

    def count_between(self, t0, t1):
        return sum(1 for t, _ in self.samples if t0 <= t <= t1)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0, t1):
        if not self.proc:
            return None
        rows = [v for t, v in self.samples if t0 <= t <= t1] or [v for _, v in self.samples]
        if not rows:
            return None

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if len(r) > 2 and num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if len(r) > 2 and num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 5 + i and "Active" in r[5 + i]
                          and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback 6.8 TB/s"


def profiled_traffic(workload):
    """Per-launch DRAM bytes of the product kernel from the committed ncu summary, if any."""
    try:
        with open(os.path.join(ROOT, "profiles", "hx_traffic.json")) as f:
            d = json.load(f)
        return d.get(workload)
    except (OSError, ValueError):
        return None


# ---------------------------------------------------------------------------------------------------
def dist_setup():
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return world, rank, local


def combine_ranks(local_seconds: float, local_bytes: float):
    """Slowest rank's time and the sum of all ranks' bytes (replicas)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return local_seconds, local_bytes
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([local_seconds], dtype=torch.float64, device=dev)
    b = torch.tensor([local_bytes], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(b, op=dist.ReduceOp.SUM)
    return float(t.item()), float(b.item())


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


# ---------------------------------------------------------------------------------------------------
def workload_config(wl, name):
    """The workload's constants, identical in both arms: sizes, exact off-diagonal nonzero count, the
    byte model of one mixed-precision H*x, and how the timing keeps x out of L2."""
    N, nnz = wl["N_r"], wl["nnz_off"]
    x_mb = N * 8 / 1e6
    if x_mb > 2 * L2_BYTES / 1e6:
        l2 = f"x alone ({x_mb:.0f} MB complex64) exceeds twice the 129 MB L2"
    else:
        l2 = "inputs cycled from a pool of x/y vectors larger than twice the 129 MB L2"
    return {"workload": name, "description": wl["desc"], "N_r": N, "nnz_off": nnz,
            "bytes_per_step": bytes_model(N, nnz, 8), "bytes_model": "N_r*(8+8+2*8) + nnz_off*(8+8)",
            "step": "one H*x over the whole sector", "l2": l2}


def _tables_restatement(wl):
    """The reference's own data structures on the host (parent basis, parent-sized mapping tables),
    for the workloads where they fit: (space, terms, N)."""
    from oracle import oracle as O
    n, bonds, jxy, jz, shape, k = hamiltonian_spec(wl)
    parent = O.popcount_basis(n, n // 2)
    terms = O.heisenberg_terms(n, bonds, jxy, jz)
    if wl["kind"] == "chain_full":
        return parent, terms, parent.size
    sites = O.spin_half_sites(n)
    bw, off = O.bit_layout(sites)
    maps, amps = O.translation_symops(shape, k)
    red = O.symmetry_reduce(parent, bw, off, maps, amps)
    return red, terms, red.dim


def cpu_tables(wl, steps, warmup, budget_s=None):
    """The reference's mul! restated on the host with its own data structures (binary search over the
    parent basis, parent-sized mapping tables, rows split statically over all host threads as
    apply_parallel! does), FP64.  A step is one whole H*x."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    space, terms, N = _tables_restatement(wl)
    setup = time.perf_counter() - t0
    x = O.complex_gaussian(N, wl["seed"])
    y = np.zeros(N, dtype=np.complex128)
    for _ in range(warmup):
        O.apply_rows(space, terms, x, out=y)
    done, tot = 0, 0.0
    while True:
        t0 = time.perf_counter()
        O.apply_rows(space, terms, x, out=y)
        tot += time.perf_counter() - t0
        done += 1
        if steps is not None and done >= steps:
            break
        if budget_s is not None and tot >= budget_s:
            break
    ms = 1e3 * tot / done
    return {"ms_per_step": ms, "steps": done, "cores": O.num_threads(), "kind": "port", "setup_s": setup,
            "sample": f"{done} whole H*x of the {N}-row sector (FP64, the reference's parent-sized tables), "
                      f"{tot:.2f} s of CPU time"}


def cpu_orbit_rows(wl, steps, warmup, budget_s=None, rows_per_step=4096):
    """The reference's row formula on the host for sectors whose parent-sized tables do not fit in host
    memory (the 6x6 torus: ~290 GB): the representatives are enumerated on the host (orbit minima with
    trivial stabiliser character, the set the reference's sweep keeps), and the mapping entries each
    row needs are evaluated orbit by orbit (oracle.OrbitTables), FP64, all host threads.  A step is a
    block of rows_per_step random rows; its time is extrapolated to one whole H*x."""
    from oracle import oracle as O
    n, bonds, jxy, jz, shape, k = hamiltonian_spec(wl)
    t0 = time.perf_counter()
    basis = O.torus_representatives(shape, n // 2, k)
    maps, amps = O.translation_symops(shape, k)
    ot = O.OrbitTables(n, n // 2, maps, amps, basis, torus=shape)   # translations applied by word rotations
    terms = O.heisenberg_terms(n, bonds, jxy, jz)
    N = basis.size
    x = O.complex_gaussian(N, wl["seed"])
    setup = time.perf_counter() - t0
    rng = np.random.default_rng(wl["seed"])
    for _ in range(warmup):
        ot.rows(terms, x, rng.integers(0, N, rows_per_step))
    done, tot = 0, 0.0
    while True:
        sample = rng.integers(0, N, rows_per_step)
        t0 = time.perf_counter()
        ot.rows(terms, x, sample)
        tot += time.perf_counter() - t0
        done += 1
        if steps is not None and done >= steps:
            break
        if budget_s is not None and tot >= budget_s:
            break
    per_row = tot / (done * rows_per_step)
    return {"ms_per_step": 1e3 * per_row * N, "steps": done, "cores": O.num_threads(), "kind": "port",
            "setup_s": setup, "N_r_host": int(N),
            "sample": f"{done} blocks of {rows_per_step} random rows of the {N}-row sector (FP64; representatives "
                      f"enumerated on the host, mapping entries evaluated orbit by orbit instead of the reference's "
                      f"parent-sized tables, ~{24 * math.comb(n, n // 2) / 1e9:.0f} GB over {math.comb(n, n // 2)} parent "
                      f"states), "
                      f"{tot:.2f} s of CPU time, extrapolated to one whole H*x"}


def cpu_reference(wl, steps, warmup, budget_s=None):
    """The CPU arm for a workload: the table-based restatement where the reference's tables fit, else
    the orbit-by-orbit restatement of the same row formula on sampled rows."""
    if wl.get("cpu_feasible", True):
        return cpu_tables(wl, steps, warmup, budget_s)
    return cpu_orbit_rows(wl, steps, warmup, budget_s)


def tridiagonal_e0_change(r, k):
    """|E0(steps) - E0(steps - k)| from a Lanczos run's coefficients (convergence of the estimate)."""
    import numpy as np
    from scipy.linalg import eigvalsh_tridiagonal
    n = r.steps
    if n <= k + 1:
        return None
    a, b = np.asarray(r.alphas[:n]), np.asarray(r.betas[:n - 1])
    e_all = eigvalsh_tridiagonal(a, b, select="i", select_range=(0, 0))[0]
    e_less = eigvalsh_tridiagonal(a[:n - k], b[:n - k - 1], select="i", select_range=(0, 0))[0]
    return float(abs(e_all - e_less))


def run_reference(args, wl):
    """The reference arm: the reference's mul! restated on the host cores, on the same workload, metric
    and config as the GPU arm.  value = the workload's bytes_per_step over the time of one whole H*x
    (so the ratio of the two arms' values is the ratio of their H*x times)."""
    world, rank = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cfg = workload_config(wl, args.workload)
    if wl["kind"] == "torus_allk":
        # the batched workload: the per-sector restatement on one momentum sector of it, scaled by the
        # sector count (all sectors have the same size to within 29 rows)
        one = dict(WORKLOADS["triangular6x5_k1"])
        r = cpu_orbit_rows(one, args.steps, args.warmup)
        r["ms_per_step"] *= 30
        r["sample"] += "; one sector (k=(1,0)) of the 30, time multiplied by 30"
    else:
        r = cpu_reference(wl, args.steps, args.warmup)
    value = cfg["bytes_per_step"] / (r["ms_per_step"] / 1e3) / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": value, "unit": "GB/s", "cores": r["cores"], "kind": r["kind"],
                             "sample": r["sample"]},
            "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "setup_s": r["setup_s"]}
    if not wl.get("cpu_feasible", True) and not args.no_cpu_baseline:
        # the reference's own data structures on the largest configuration where they fit in seconds
        t = cpu_tables(WORKLOADS["chain24_k0"], None, 1, budget_s=args.cpu_seconds)
        c24 = workload_config(WORKLOADS["chain24_k0"], "chain24_k0")
        t["value"] = c24["bytes_per_step"] / (t["ms_per_step"] / 1e3) / 1e9
        t["unit"] = "GB/s"
        t["config"] = c24
        line["cpu_reference_tables_chain24_k0"] = t
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------------------
def run_gpu(args, wl):
    import numpy as np
    import torch
    import edgpu

    world, rank, local = dist_setup()
    dev = torch.cuda.current_device()
    space, opr, t_space = build_gpu_operator(wl)
    N = space.dimension
    n_targets, nnz = opr.count_nnz()
    if N != wl["N_r"] or (wl["nnz_off"] is not None and nnz != wl["nnz_off"]):
        raise RuntimeError(f"sector size {N} / nonzeros {nnz} differ from the workload's {wl['N_r']} / {wl['nnz_off']}")
    cfg = workload_config(dict(wl, nnz_off=nnz), args.workload)
    dir_stats = edgpu.search_stats(space)
    map_info = build_maps([space], args)
    table_info = build_tables([opr], [space], args)
    slab_info = build_slabs(opr, N, args) if table_info and table_info.get("built") else None
    if args.no_pair:
        opr.set_pair_schedule(False)
    if args.tiling:
        # a fixed schedule instead of the autotuner (reproducible profiles); the slab table when built
        opr.set_pair_schedule(args.pair_targets > 0, max(args.pair_targets, 2), args.uniform)
        for prec in ("mixed", "fp64"):
            opr.set_tiling(prec, args.tiling)
            opr.table_prefetch(prec, args.prefetch)
            if slab_info and slab_info.get("built"):
                opr.slab_use(prec, args.slab_mode)
        tune_mixed = tune_fp64 = (args.tiling, None)
    else:
        tune_mixed = opr.autotune("mixed")
        tune_fp64 = opr.autotune("fp64")
    if slab_info and slab_info.get("built") and opr.slab_use("mixed") and opr.slab_use("fp64") and \
            not args.keep_targets:
        # both precisions read the slab table: the target table (75 GB on 6x6) is only kept for the
        # autotuner, and its memory goes to the Krylov basis of the E0 runs
        opr.free_targets()
        table_info["freed_after_slabs"] = True
    stream = torch.cuda.current_stream()

    def pool(prec):
        s_c = 8 if prec == "mixed" else 16
        P = max(2, min(4096, math.ceil(2 * L2_BYTES / (2 * N * s_c))))
        xs = [edgpu.random_state(N, wl["seed"] * 1000 + i, prec) for i in range(P)]
        ys = [torch.empty_like(xs[0]) for _ in range(P)]
        return xs, ys, P, s_c

    def timed(prec, steps, warmup):
        """K steps captured once into a CUDA graph, then replayed between CUDA events on this stream."""
        xs, ys, P, s_c = pool(prec)
        for i in range(warmup):
            edgpu.mul_(ys[i % P], opr, xs[i % P], precision=prec)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            for i in range(steps):
                edgpu.mul_(ys[i % P], opr, xs[i % P], precision=prec)
        graph.replay()                      # untimed: uploads the graph
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t_wall0 = time.time()
        e0.record(stream)
        graph.replay()
        e1.record(stream)
        torch.cuda.synchronize()
        t_wall1 = time.time()
        barrier()
        return e0.elapsed_time(e1), P, s_c, (t_wall0, t_wall1), graph

    clocks = ClockSampler(dev) if rank == 0 else None
    ms_mixed, P_mixed, s_c, (tw0, tw1), graph = timed("mixed", args.steps, args.warmup)
    # keep the GPU busy with the same graph until the clock sampler has seen the load
    if clocks and clocks.proc:
        t_end = time.time() + 2.0
        while clocks.count_between(tw0, time.time()) < 3 and time.time() < t_end:
            graph.replay()
            torch.cuda.synchronize()
        tw1 = max(tw1, time.time())
    del graph
    clk = clocks.summary(tw0 - 0.15, tw1 + 0.15) if clocks else None
    if clocks:
        clocks.stop()

    b_mixed = bytes_model(N, nnz, 8)
    t_max, b_all = combine_ranks(ms_mixed / 1e3, b_mixed * args.steps)
    value = b_all / t_max / 1e9
    per_launch_ms = ms_mixed / args.steps
    achieved = b_mixed / (per_launch_ms / 1e3) / 1e9

    fp64_steps = max(1, args.steps // 4)
    ms64, _, _, _, graph64 = timed("fp64", fp64_steps, max(3, args.warmup // 4))
    del graph64
    b64 = bytes_model(N, nnz, 16)
    value64 = b64 / (ms64 / fp64_steps / 1e3) / 1e9

    # end to end through the C ABI with host complex128 buffers (the reference's mul! interface on
    # Vector{ComplexF64}): pinned buffers (graph-replayed, kernels address the host buffers), and the
    # ordinary pageable buffers a Julia ccall passes (copies through the library's device buffers)
    x_h = torch.empty(N, dtype=torch.complex128, pin_memory=True)
    y_h = torch.empty(N, dtype=torch.complex128, pin_memory=True)
    x_h.copy_(edgpu.random_state(N, wl["seed"], "fp64").cpu())
    xn, yn = x_h.numpy(), y_h.numpy()
    e2e_steps = max(3, min(args.steps, 500))

    def host_timed(xa, ya, prec, k):
        for _ in range(2):
            edgpu.mul_(ya, opr, xa, precision=prec)
        barrier()
        t0 = time.perf_counter()
        for _ in range(k):
            edgpu.mul_(ya, opr, xa, precision=prec)
        return (time.perf_counter() - t0) / k

    t_e2e = host_timed(xn, yn, "mixed", e2e_steps)
    e2e = {"value": b_mixed / t_e2e / 1e9, "unit": "GB/s", "h2d_bytes_per_step": 16 * N, "d2h_bytes_per_step": 16 * N,
           "ms_per_step": t_e2e * 1e3, "buffers": "pinned complex128", "product": "mixed"}
    t_e2e64 = host_timed(xn, yn, "fp64", max(3, e2e_steps // 4))
    xp, yp = np.array(xn), np.empty_like(xn)          # pageable copies
    t_pg = host_timed(xp, yp, "mixed", max(3, e2e_steps // 4))
    del xp, yp
    # the host link itself: plain pinned copies of the same bytes each way (cudaMemcpyAsync)
    dbuf = torch.empty(N, dtype=torch.complex128, device="cuda")
    for _ in range(2):
        dbuf.copy_(x_h, non_blocking=True)
    torch.cuda.synchronize()
    e0_, e1_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0_.record()
    for _ in range(3):
        dbuf.copy_(x_h, non_blocking=True)
    e1_.record()
    torch.cuda.synchronize()
    h2d = 3 * 16 * N / (e0_.elapsed_time(e1_) / 1e3) / 1e9
    e0_.record()
    for _ in range(3):
        y_h.copy_(dbuf, non_blocking=True)
    e1_.record()
    torch.cuda.synchronize()
    d2h = 3 * 16 * N / (e0_.elapsed_time(e1_) / 1e3) / 1e9
    del dbuf
    host_link = {"h2d_gbs": h2d, "d2h_gbs": d2h, "bytes_each_way": 16 * N,
                 "copy_only_ms": 16 * N / h2d / 1e6 + 16 * N / d2h / 1e6}
    e2e_more = {"fp64_pinned": {"value": b_mixed / t_e2e64 / 1e9, "ms_per_step": t_e2e64 * 1e3},
                "mixed_pageable": {"value": b_mixed / t_pg / 1e9, "ms_per_step": t_pg * 1e3}}

    # time to E0 (Lanczos): FP64 product vs mixed product polished in FP64
    e0_info = None
    if not args.no_lanczos:
        # Time to E0.  The FP64 oracle: FP64 Lanczos from the seeded start vector until the lowest Ritz
        # value settles to 1e-12 relative over five steps.  Against the 1e-9 target both arms then run to
        # 1e-10: FP64 Lanczos (settled to 1e-10), and mixed-precision Lanczos (complex64 products, settled
        # to 1e-9) followed by the FP64 Rayleigh quotient of its Ritz vector, accepted when the
        # Kato-Temple estimate of its error is below 1e-10 relative (else FP64 Lanczos from that vector).
        # the stored Krylov basis (which gives the Ritz vector without a second pass of the recurrence)
        # may take the device memory left after the operator's tables (the Lanczos driver sizes it after
        # its other buffers and keeps 2 GiB free)
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        free_b, _ = torch.cuda.mem_get_info()
        krylov_limit = int(free_b)
        edgpu.set_krylov_limit(krylov_limit)
        t0 = time.perf_counter()
        r64 = edgpu.lanczos(opr, wl["lanczos_steps"], precision="fp64", reorth=wl["reorth"], seed=wl["seed"], tol=1e-12)
        t64 = time.perf_counter() - t0
        t0 = time.perf_counter()
        r64b = edgpu.lanczos(opr, wl["lanczos_steps"], precision="fp64", reorth=wl["reorth"], seed=wl["seed"], tol=1e-10)
        t64b = time.perf_counter() - t0
        t0 = time.perf_counter()
        rmx = edgpu.lanczos(opr, wl["lanczos_steps"], precision="mixed", reorth=wl["reorth"], seed=wl["seed"],
                            refine=True, tol=1e-10)
        tmx = time.perf_counter() - t0
        e0_info = {"fp64_oracle_s": t64, "fp64_s": t64b, "mixed_s": tmx, "target_rel": 1e-9, "tol": 1e-10,
                   "e0_fp64_oracle": r64.e0, "e0_fp64": r64b.e0, "e0_mixed": rmx.e0,
                   "rel_diff": abs(rmx.e0 - r64.e0) / abs(r64.e0),
                   "rel_diff_fp64": abs(r64b.e0 - r64.e0) / abs(r64.e0),
                   "steps_fp64_oracle": r64.steps, "steps_fp64": r64b.steps, "steps_mixed": rmx.steps,
                   "reorth": bool(wl["reorth"]), "max_steps": wl["lanczos_steps"], "krylov_limit_bytes": krylov_limit,
                   "fp64_e0_change_last_20_steps": tridiagonal_e0_change(r64, 20)}
        edgpu.set_krylov_limit(0)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and wl["kind"] != "torus_pg":
        r = cpu_reference(wl, None, 1, budget_s=args.cpu_seconds)
        cpu = {"value": cfg["bytes_per_step"] / (r["ms_per_step"] / 1e3) / 1e9, "unit": "GB/s", "cores": r["cores"],
               "kind": r["kind"], "sample": r["sample"], "ms_per_step": r["ms_per_step"]}

    peak, peak_src = measured_peak()
    slab_used = bool(slab_info and slab_info.get("built") and opr.slab_use("mixed"))
    # DRAM bytes per step of the product as profiled: the slab product's passes, or the one-pass kernel
    traffic = profiled_traffic(args.workload + ("_slabs" if slab_used else ""))
    # one launch per slab pass, and on a scaled slab table one scaling of x per pass
    launches_per_step = slab_info["passes"] * (2 if slab_info.get("scaled") else 1) if slab_used else 1
    line = {"metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": cfg,
            "gpu_setup": {"n_targets": n_targets, "pool": f"{P_mixed} x/y pairs ({2 * P_mixed * N * s_c / 1e6:.0f} MB)",
                       "parallelism": f"replicas x{world}",
                       "rows_per_tile": {"mixed": tune_mixed[0], "fp64": tune_fp64[0]},
                       "pair_flip_schedule": {"mixed": opr.schedule("mixed")[1], "fp64": opr.schedule("fp64")[1],
                                              "bond_classes": opr.pair_classes()[0],
                                              "prefetch": {"mixed": opr.table_prefetch("mixed"),
                                                           "fp64": opr.table_prefetch("fp64")}},
                       "target_table": dict(table_info or {"built": False},
                                            used={"mixed": opr.uses_target_table("mixed"),
                                                  "fp64": opr.uses_target_table("fp64")}),
                       "slab_table": dict(slab_info or {"built": False},
                                          used={"mixed": opr.slab_use("mixed") if slab_info and slab_info.get("built") else 0,
                                                "fp64": opr.slab_use("fp64") if slab_info and slab_info.get("built") else 0},
                                          use_codes="0 none, 1 slab product, 2 with cache hints, 3 eight entries "
                                                    "per step, 4 both, 5 two lanes per row, 6 four lanes per row"),
                       "setup_s": t_space, "search_directory": dir_stats, "parent_map": map_info},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "peak_source": peak_src,
                         "scope": f"one H*x ({launches_per_step} launch{'es' if launches_per_step > 1 else ''}): "
                                  "model bytes over its device time; traffic = DRAM bytes of one H*x from the "
                                  "committed ncu summary"},
            "cpu_baseline": cpu, "e2e": e2e, "e2e_more": e2e_more, "host_link": host_link,
            "gpu_launches": args.steps * launches_per_step, "clocks": clk,
            "fp64": {"value": value64, "unit": "GB/s", "ms_per_step": ms64 / fp64_steps, "frac": value64 / peak},
            "e0": e0_info}
    if rank == 0:
        print(json.dumps(line), flush=True)
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()


def run_gpu_batch(args, wl):
    """All momentum sectors of one Hamiltonian in one persistent launch per step (edgpu_batch_*)."""
    import torch
    import edgpu

    world, rank, local = dist_setup()
    dev = torch.cuda.current_device()
    spaces, oprs, momenta, t_space = build_gpu_sectors(wl)
    dims = [sp.dimension for sp in spaces]
    N = sum(dims)
    nnz = sum(o.count_nnz()[1] for o in oprs)
    if N != wl["N_r"] or (wl["nnz_off"] is not None and nnz != wl["nnz_off"]):
        raise RuntimeError(f"sector sizes {N} / nonzeros {nnz} differ from the workload's {wl['N_r']} / {wl['nnz_off']}")
    cfg = workload_config(dict(wl, nnz_off=nnz), args.workload)
    map_info = build_maps(spaces, args)
    table_info = build_tables(oprs, spaces, args)
    slab_info = None
    if table_info and table_info.get("built") and args.slab_mb > 0:
        # every sector's slab table (the batch autotuner times per-sector launches through them)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        slab_info = {"built": True, "passes": [], "entries": 0}
        for o in oprs:
            free, _ = torch.cuda.mem_get_info()
            o.slab_scaling(args.slab_scaling)
            if not o.build_slabs(slab_bytes=int(args.slab_mb * (1 << 20)), max_bytes=int(0.5 * free)):
                slab_info = {"built": False}
                break
            slab_info["passes"].append(o.slabs_info[0])
            slab_info["entries"] += o.slabs_info[2]
            slab_info["scaled_sectors"] = slab_info.get("scaled_sectors", 0) + int(o.slab_scaling())
        if slab_info["built"]:
            slab_info["passes"] = sorted(set(slab_info["passes"]))
        slab_info["build_s"] = time.perf_counter() - t0
    if args.no_pair:
        for o in oprs:
            o.set_pair_schedule(False)
    batch = edgpu.Batch(oprs)
    if args.tiling:
        # a fixed schedule for every sector and a fixed batch launch mode instead of the autotuners
        # (reproducible profiles)
        for o in oprs:
            o.set_pair_schedule(args.pair_targets > 0, max(args.pair_targets, 2), args.uniform)
            o.set_tiling("mixed", args.tiling)
            o.table_prefetch("mixed", args.prefetch)
            if slab_info and slab_info.get("built"):
                o.slab_use("mixed", args.slab_mode)
        batch.set_launch("mixed", args.batch_launch)
        lpr, tune_ms = -args.tiling, None
    else:
        # each sector's own schedule first (the batch autotuner also times per-sector launches with them)
        for o in oprs:
            o.autotune("mixed")
        lpr, tune_ms = batch.autotune("mixed")
    stream = torch.cuda.current_stream()
    s_c = 8
    P = max(2, math.ceil(2 * L2_BYTES / (2 * N * s_c)))
    sets = []
    for i in range(P):
        xs = [edgpu.random_state(d, wl["seed"] * 1000 + 100 * i + j, "mixed") for j, d in enumerate(dims)]
        sets.append((xs, [torch.empty_like(x) for x in xs]))
    for i in range(max(args.warmup, P)):                 # uploads each pointer set's sector descriptors
        xs, ys = sets[i % P]
        batch.mul_(ys, xs, precision="mixed", use_graph=False)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        for i in range(args.steps):
            xs, ys = sets[i % P]
            batch.mul_(ys, xs, precision="mixed", use_graph=False)
    graph.replay()
    torch.cuda.synchronize()
    clocks = ClockSampler(dev) if rank == 0 else None
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    tw0 = time.time()
    if args.profile_range:
        torch.cuda.profiler.start()       # a profiler started with --profile-from-start off sees this only
    e0.record(stream)
    graph.replay()
    e1.record(stream)
    torch.cuda.synchronize()
    if args.profile_range:
        torch.cuda.profiler.stop()
    tw1 = time.time()
    barrier()
    ms = e0.elapsed_time(e1)
    if clocks and clocks.proc:
        t_end = time.time() + 2.0
        while clocks.count_between(tw0, time.time()) < 3 and time.time() < t_end:
            graph.replay()
            torch.cuda.synchronize()
        tw1 = max(tw1, time.time())
    del graph
    clk = clocks.summary(tw0 - 0.15, tw1 + 0.15) if clocks else None
    if clocks:
        clocks.stop()
    b_step = bytes_model(N, nnz, s_c)
    t_max, b_all = combine_ranks(ms / 1e3, b_step * args.steps)
    # kernel launches of one batched product: one persistent launch, or per sector one launch (its
    # slab product: one per slab)
    mode = batch.launch("mixed")
    if mode == 0:
        launches_per_step = 1
    elif mode >= 5:
        launches_per_step = sum((o.slabs_info[0] * (2 if o.slab_scaling() else 1) if o.slab_use("mixed") else 1)
                                for o in oprs if o.dimension)
    else:
        launches_per_step = sum(1 for o in oprs if o.dimension)
    value = b_all / t_max / 1e9
    achieved = b_step / (ms / args.steps / 1e3) / 1e9

    # the same sectors as separate products, each operator with its own autotuned schedule, launched
    # one after the other on one stream (what a caller without the batch would do)
    per_sector_ms = None
    if not args.no_per_sector:
        xs, ys = sets[0]
        for o, x, y in zip(oprs, xs, ys):
            edgpu.mul_(y, o, x, precision="mixed")
        torch.cuda.synchronize()
        ps_steps = max(3, min(args.steps, 10))
        e0.record(stream)
        for i in range(ps_steps):
            xs, ys = sets[i % P]
            for o, x, y in zip(oprs, xs, ys):
                edgpu.mul_(y, o, x, precision="mixed")
        e1.record(stream)
        torch.cuda.synchronize()
        per_sector_ms = e0.elapsed_time(e1) / ps_steps

    # library graph path (the call a user makes: captured once per pointer set, replayed)
    xs, ys = sets[0]
    batch.mul_(ys, xs, precision="mixed", use_graph=True)
    torch.cuda.synchronize()
    g_steps = max(3, min(args.steps, 50))
    e0.record(stream)
    for _ in range(g_steps):
        batch.mul_(ys, xs, precision="mixed", use_graph=True)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_graph = e0.elapsed_time(e1) / g_steps

    # end to end with pinned host complex64 vectors: copies in, one batched product, copies out
    xh = [torch.empty(d, dtype=torch.complex64, pin_memory=True) for d in dims]
    yh = [torch.empty(d, dtype=torch.complex64, pin_memory=True) for d in dims]
    for h, x in zip(xh, sets[0][0]):
        h.copy_(x.cpu())
    e2e_steps = max(3, min(args.steps, 20))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for h, x in zip(xh, xs):
            x.copy_(h, non_blocking=True)
        batch.mul_(ys, xs, precision="mixed", use_graph=True)
        for h, y in zip(yh, ys):
            h.copy_(y, non_blocking=True)
        torch.cuda.synchronize()
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    e2e = {"value": b_step / t_e2e / 1e9, "unit": "GB/s", "h2d_bytes_per_step": 8 * N, "d2h_bytes_per_step": 8 * N,
           "ms_per_step": t_e2e * 1e3}

    peak, peak_src = measured_peak()
    line = {"metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": cfg,
            "gpu_setup": {"sectors": len(dims), "N_r_min": min(dims), "N_r_max": max(dims),
                       "lanes_per_row": lpr, "pair_flip_schedule": batch.schedule("mixed")[1],
                       "target_table": dict(table_info or {"built": False}, used=batch.uses_target_tables("mixed")),
                       "bond_classes": oprs[0].pair_classes()[0], "l2": f"inputs cycled from {P} sets of x/y ({2 * P * N * s_c / 1e6:.0f} MB "
                       f"> 2x L2)", "parallelism": f"replicas x{world}", "setup_s": t_space,
                       "library_graph_ms_per_step": ms_graph, "parent_map": map_info, "slab_tables": slab_info,
                       "batch_launch": {0: "one persistent launch"}.get(
                           batch.launch("mixed"), f"per-sector launches on {batch.launch('mixed') & 3} stream(s)" +
                           (", each sector with its own autotuned schedule" if batch.launch("mixed") >= 5 else "")),
                       "per_sector_launches_ms_per_step": per_sector_ms},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": profiled_traffic(args.workload), "peak_source": peak_src,
                         "scope": "one batched H*x over all sectors (all its launches); traffic = DRAM bytes of one "
                                  "batched H*x from the committed ncu summary"},
            "cpu_baseline": None if args.no_cpu_baseline else
            {"value": None, "unit": "GB/s", "cores": None, "kind": "port",
             "sample": "not run: the reference builds a 155M-state parent basis and 3.7 GB of mapping tables per sector"},
            "e2e": e2e, "gpu_launches": args.steps * launches_per_step, "clocks": clk}
    line["gpu_setup"]["launches_per_step"] = launches_per_step
    if rank == 0:
        print(json.dumps(line), flush=True)
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()


def run_gpu_grad(args, wl):
    """Forward product, fused coupling gradient and adjoint product of a per-bond-coupling chain."""
    import numpy as np
    import torch
    import edgpu
    from edgpu import lattice

    world, rank, local = dist_setup()
    dev = torch.cuda.current_device()
    L = wl["L"]
    hs, _ = edgpu.spin_half_system(L)
    t0 = time.perf_counter()
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0), lazy=True)
    space = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, wl["k"]))
    t_space = time.perf_counter() - t0
    J = 0.5 + np.random.default_rng(wl["seed"]).random(L)
    m, r, c, a, ids = lattice.heisenberg_coupled(hs, lattice.chain_bonds(L))
    opr = edgpu.OperatorRepresentation.from_terms(space, m, r, c, a, coupling_ids=ids, couplings=J)
    N = space.dimension
    n_targets, nnz = opr.count_nnz()
    if N != wl["N_r"] or (wl["nnz_off"] is not None and nnz != wl["nnz_off"]):
        raise RuntimeError(f"sector size {N} / nonzeros {nnz} differ from the workload's {wl['N_r']} / {wl['nnz_off']}")
    cfg = workload_config(dict(wl, nnz_off=nnz), args.workload)
    map_info = build_maps([space], args)
    table_info = build_tables([opr], [space], args)
    # the column-sorted adjoint table: the adjoint of these (non-invariant) terms as a gather in a fixed order
    adjoint_table = bool(table_info and table_info.get("built")) and opr.build_adjoint_targets()
    # the slab table for the forward product (the gradient and the adjoint have their own kernels)
    slab_info = build_slabs(opr, N, args) if table_info and table_info.get("built") else None
    opr.autotune("mixed")
    opr.autotune("fp64")
    stream = torch.cuda.current_stream()
    res = {}
    for prec in ("mixed", "fp64"):
        x = edgpu.random_state(N, wl["x_seed"], prec)
        gy = edgpu.random_state(N, wl["gy_seed"], prec)
        y = torch.empty_like(x)
        gx = torch.empty_like(x)
        for _ in range(args.warmup):
            edgpu.mul_(y, opr, x, precision=prec)
            edgpu.coupling_grad(opr, x, gy, precision=prec, y=y)
            edgpu.mul_adjoint_(gx, opr, gy, precision=prec)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        times = {}
        for name, fn in (("forward", lambda: edgpu.mul_(y, opr, x, precision=prec)),
                         ("forward_and_coupling_grad", lambda: edgpu.coupling_grad(opr, x, gy, precision=prec, y=y)),
                         ("adjoint", lambda: edgpu.mul_adjoint_(gx, opr, gy, precision=prec))):
            barrier()
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(args.steps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            times[name] = e0.elapsed_time(e1) / args.steps
        res[prec] = times
    b = bytes_model(N, nnz, 8)
    t_fwd = res["mixed"]["forward"] / 1e3
    t_max, b_all = combine_ranks(t_fwd * args.steps, b * args.steps)
    peak, peak_src = measured_peak()
    line = {"metric": METRIC, "value": b_all / t_max / 1e9, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": cfg,
            "gpu_setup": {"invariant_terms": opr.is_invariant, "setup_s": t_space, "parent_map": map_info,
                          "target_table": table_info, "adjoint_table": adjoint_table,
                          "slab_table": dict(slab_info or {"built": False},
                                             forward_uses={p: opr.slab_use(p) for p in ("mixed", "fp64")}
                                             if slab_info and slab_info.get("built") else None),
                          "grad_kernel": {"mixed": opr.grad_kernel("mixed"), "fp64": opr.grad_kernel("fp64")},
                          "ms": res, "parallelism": f"replicas x{world}"},
            "roofline": {"bound": "hbm", "achieved": b / t_fwd / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": b / t_fwd / 1e9 / peak, "traffic": None, "peak_source": peak_src},
            "cpu_baseline": None, "e2e": None, "gpu_launches": args.steps, "clocks": None}
    if rank == 0:
        print(json.dumps(line), flush=True)
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed steps (default: the workload's, ~3-60 s)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="square6x6_k0")
    ap.add_argument("--no-lanczos", action="store_true")
    ap.add_argument("--no-map", action="store_true", help="canonicalise targets instead of using parent-state maps")
    ap.add_argument("--map-bytes", type=int, default=0,
                    help="byte limit of each parent-state map (0: the library default); below the direct map's "
                         "size the map is rank-indexed")
    ap.add_argument("--tiling", type=int, default=0,
                    help="fixed schedule instead of the autotuner: -1/-2/-4 lanes per row (single-sector workloads)")
    ap.add_argument("--pair-targets", type=int, default=2, choices=[0, 2, 4, 8],
                    help="with --tiling: targets per lane and step of the pair-flip schedule (0: term scan)")
    ap.add_argument("--uniform", action="store_true", help="with --tiling: warp-uniform pair steps (4 or 8 targets)")
    ap.add_argument("--prefetch", type=int, default=0, help="with --tiling: x prefetch distance of the target-table product")
    ap.add_argument("--no-table", action="store_true", help="no target tables (look every target up per product)")
    ap.add_argument("--keep-targets", action="store_true",
                    help="keep the target table when both precisions read the slab table")
    ap.add_argument("--profile-range", action="store_true",
                    help="batched workload: bracket the timed steps with cudaProfilerStart/Stop (for a "
                         "profiler run with --profile-from-start off: the autotuners run unprofiled)")
    ap.add_argument("--batch-launch", type=int, default=7, choices=[0, 1, 2, 3, 5, 6, 7],
                    help="batched workload with --tiling: the batch launch mode (edgpu_batch_set_launch)")
    ap.add_argument("--slab-mode", type=int, default=1, choices=[1, 2, 3, 4, 5, 6],
                    help="with --tiling: the slab product's variant (1 plain, 2 cache hints, 3 eight entries "
                         "per step, 4 both, 5 two lanes per row, 6 four lanes per row)")
    ap.add_argument("--slab-scaling", type=int, default=0, choices=[0, 1, 2],
                    help="slab table layout (edgpu_op_slab_scaling): 0 scaled on sectors of 2^22 rows or more "
                         "where that saves passes or the coefficients are complex, 1 never, 2 always")
    ap.add_argument("--slab-mb", type=float, default=112.0,
                    help="column slabs of this many MB of complex64 x (0: no slab table)")
    ap.add_argument("--no-pair", action="store_true", help="test every term per row instead of the pair-flip schedule")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-per-sector", action="store_true",
                    help="batched workload: skip timing the sectors as separate products")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    wl = WORKLOADS[args.workload]
    if args.steps is None:
        args.steps = wl["steps"]
    args.workload_no_map = bool(wl.get("no_map", False))
    if args.impl == "reference" and wl["nnz_off"] is None:
        if int(os.environ.get("RANK", "0")) == 0:
            print(json.dumps({"impl": "reference", "unavailable": f"{args.workload} is a profiling case without "
                                                                  "a fixed nonzero count for the byte model"}))
    elif args.impl == "reference" and wl["kind"] == "torus_pg":
        if int(os.environ.get("RANK", "0")) == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the reference builds this sector from its "
                              "9.1e9-state parent basis (~218 GB of mapping tables); the host has no enumeration "
                              "of the 288-element group's representatives without it"}))
    elif args.impl == "reference":
        run_reference(args, wl)
    elif wl["kind"] == "torus_allk":
        run_gpu_batch(args, wl)
    elif wl["kind"] == "chain_grad":
        run_gpu_grad(args, wl)
    else:
        run_gpu(args, wl)


if __name__ == "__main__":
    main()
