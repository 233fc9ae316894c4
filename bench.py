#!/usr/bin/env python
"""Benchmark of the FP64 tangent + residual assembly (Florence's low-level displacement-formulation
assembly) on one GB300.

Workload (default): the unstructured p=3 (20-node) tetrahedral mesh of a 4x1x1 beam, seeded
jittered lattice (48x12x12 cells, jitter 0.15 h, default_rng(1)) split by Delaunay, Mooney-Rivlin
mu1 = mu2 = 0.5, lambda = 20, 14 Gauss points per element, at a seeded first-increment state
(downward bending u_z = -0.02 (x/4)^2 plus three seeded smooth modes, default_rng(2)). One step =
zero the CSR values and the residual, assemble the tangent (CSR through the element-to-nonzero
maps) and the residual: one pass of the hot path.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference] [--workload beam|cube]

``--impl reference`` times the reference algorithm's CPU implementation (the C restatement of
_GlobalAssemblyDF_ in oracle/, all host threads) on the same workload and prints its own line.
Prints one JSON line.
"""
import argparse
import json
import os
import re
import subprocess
import sys
import tempfile
import threading
import time
import types

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")


# ------------------------------------------------------------------------------------------------
# workloads
# ------------------------------------------------------------------------------------------------
def workload(name):
    from florence_gb300 import meshes
    if name in ("beam", "beam_s"):
        # beam_s: the same beam at half the lattice resolution (profiling case, ~6k elements)
        t = np.load(os.path.join(GOLDEN, "tet_p3_mr_jitter.npz"))
        pat = meshes.local_pattern(t["points"], t["elements"], 0, "tet")
        cells = (48, 12, 12) if name == "beam" else (24, 6, 6)
        P, el = meshes.jittered_tet_beam(cells, (4.0, 1.0, 1.0), 1, pat)
        x = P + smooth_displacement(P, seed=2)
        desc = dict(workload="tet p=3 beam 4x1x1 (%dx%dx%d jittered lattice, Delaunay), Mooney-Rivlin "
                             "mu1=mu2=0.5 lambda=20, 14 Gauss points, FP64 tangent (CSR) + residual" % cells,
                    element="tet20", material="MooneyRivlin")
        return dict(points=P, elements=el, x=x, Jm=t["Jm"], w=t["AllGauss"], material="MooneyRivlin",
                    params=(0.5, 0.5, 20.0), desc=desc)
    if name == "cube":
        d = np.load(os.path.join(GOLDEN, "config1_hex8_p2_q5.npz"))
        desc = dict(workload="structured 8x8x8 p=2 hex cube (27-node), Gauss 5^3 = 125 points, neo-Hookean "
                             "mu=1 lambda=10, u~U(-0.01,0.01) default_rng(0), FP64 tangent (CSR) + residual",
                    element="hex27", material="NeoHookean")
        return dict(points=d["points"], elements=d["elements"], x=d["Eulerx"], Jm=d["Jm"], w=d["AllGauss"],
                    material="NeoHookean", params=(1.0, 10.0), desc=desc)
    raise ValueError(name)


def smooth_displacement(P, seed):
    """First-increment state of the beam: downward bending u_z = -0.02 (x/4)^2 plus three seeded
    Fourier modes of amplitude 2e-3 (|grad u| < 0.05, so det F > 0 on every element, slivers
    included)."""
    rng = np.random.default_rng(seed)
    u = np.zeros_like(P)
    u[:, 2] = -0.02 * (P[:, 0] / 4.0) ** 2
    for _ in range(3):
        k = rng.uniform(-2.0 * np.pi, 2.0 * np.pi, 3)
        phase = rng.uniform(0.0, 2.0 * np.pi)
        amp = rng.uniform(-2e-3, 2e-3, 3)
        u += np.sin(P @ k + phase)[:, None] * amp[None, :]
    return u


def flops_alg(npe, nq, material):
    """Algorithmic FP64 FLOPs per element of the tangent + residual, nq (6 ndof^2 + 288 npe + c),
    c = 300 (neo-Hookean) / 500 (Mooney-Rivlin): folded constitutive+geometric tensor contracted
    with the spatial gradients, kinematics, residual and material per Gauss point."""
    ndof = 3 * npe
    return nq * (6 * ndof * ndof + 288 * npe + (300 if material == "NeoHookean" else 500))


def flops_executed(npe, nq, material):
    """FP64 FLOPs the kernel executes per element (symmetric tangent: node blocks a <= b only):
    per Gauss point 27 npe (npe+1) (stiffness) + 162 npe (U) + 36 npe (kinematics) + 18 npe
    (residual) + c, c = 800 (neo-Hookean) / 1200 (Mooney-Rivlin)."""
    return nq * (27 * npe * (npe + 1) + 216 * npe + (800 if material == "NeoHookean" else 1200))


EPC = {4: 8, 8: 8, 10: 4, 20: 2, 27: 1, 35: 1, 64: 1, 125: 1}   # elements per CTA of the contraction


def assembly_launches(nelem, npe, nq):
    """Kernels one assembly call launches: (Gauss-point kernel + contraction) per chunk of the
    64 MiB Gauss-point scratch (54 doubles per Gauss point)."""
    ce = (64 << 20) // (8 * 54 * nq)
    ce -= ce % EPC[npe]
    return 2 * ((nelem + ce - 1) // ce)


def mixed_launches(nelem, nq):
    """Kernels one split-BF16 assembly call launches: the float4 table of the shape-function
    gradients, then (Gauss-point kernel + contraction) per chunk of the 64 MiB Gauss-point scratch
    (9 doubles + 45 floats per Gauss point)."""
    ce = max(1, (64 << 20) // ((9 * 8 + 45 * 4) * nq))
    return 1 + 2 * ((nelem + ce - 1) // ce)


def tensor_launches(nelem, nq):
    """Kernels one FP64 tensor-core assembly call launches: the float-pair table of the
    shape-function gradients, then (Gauss-point kernel + contraction) per chunk of the 64 MiB
    Gauss-point scratch (9 doubles + 90 floats per Gauss point)."""
    ce = max(1, (64 << 20) // ((9 * 8 + 90 * 4) * nq))
    return 1 + 2 * ((nelem + ce - 1) // ce)


def rt_launches(nelem, nq):
    """Kernels one reference-tensor assembly call launches (block offsets kept by the assembler):
    the float-pair node and shape-function tables, the reference tensor's digit planes, then
    (Gauss-point kernel + contraction) per chunk of at most 512 MB of Gauss-point data."""
    ce = max(1, (512 << 20) // (8 * 54 * nq))
    return 3 + 2 * ((nelem + ce - 1) // ce)


def pair_macs(npe, nq):
    """Multiply-adds of the contraction per element (stiffness node blocks a <= b and the U
    build), each 12 FP32-pipe instructions in the float-pair arithmetic."""
    return nq * (27 * npe * (npe + 1) // 2 + 81 * npe)


def bytes_min(nnode, nelem, npe, nnz):
    """Compulsory HBM bytes of one assembly: X and x read, connectivity (int32 equivalent), CSR
    values written once, residual written."""
    return 8 * 3 * nnode * 2 + 4 * nelem * npe + 8 * nnz + 8 * 3 * nnode


# ------------------------------------------------------------------------------------------------
# clocks
# ------------------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.proc = None
        self.out = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        self.out.flush()
        rows = []
        with open(self.out.name) as f:
            for line in f:
                p = [c.strip() for c in line.split(",")]
                if len(p) >= 7:
                    try:
                        rows.append((float(p[0]), float(p[1]), p[3:7]))
                    except ValueError:
                        pass
        os.unlink(self.out.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower().startswith("active")})
        return {"sm_mhz": float(np.median([r[0] for r in rows])), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def traffic_from_profile(kernel_tag):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", kernel_tag + ".md")
    if not os.path.exists(path):
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", open(path).read())
    return float(m.group(1)) if m else None


def bench_config(W, nnz, world=1):
    """The `config` object of both arms' lines (identical keys and values for one workload)."""
    nelem = int(W["elements"].shape[0])
    nq = int(np.ravel(W["w"]).shape[0])
    nnode = int(W["points"].shape[0])
    return dict(W["desc"], nelem=nelem, nnode=nnode, nnz=int(nnz), gauss_points=nq,
                parallelism="replicas" if world > 1 else "single GPU",
                l2="inputs larger than L2: CSR values %.0f MB and element-to-nonzero map %.0f MB per step"
                   % (nnz * 8 / 1e6, nelem * (3 * W["elements"].shape[1]) ** 2 * 4 / 1e6))


def cpu_model():
    """Model string of the host CPU (lscpu, else /proc/cpuinfo, else the platform module)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


# ------------------------------------------------------------------------------------------------
# CPU reference (oracle restatement of _GlobalAssemblyDF_)
# ------------------------------------------------------------------------------------------------
def one_core_rate(W, sample_elems=6000, passes=3):
    """Melem/s of the C restatement on one thread, on the first `sample_elems` elements of the
    workload (renumbered to the nodes they use, their own CSR pattern), best of `passes`."""
    from oracle import oracle
    el = W["elements"][:sample_elems]
    used, inv = np.unique(el, return_inverse=True)
    el = inv.reshape(el.shape).astype(np.int64)
    P, x = W["points"][used], W["x"][used]
    spa = oracle.sparsity(el, P.shape[0])
    times = []
    for _ in range(passes):
        t0 = time.perf_counter()
        oracle.assemble_df(W["material"], W["params"], P, el, x, W["Jm"], W["w"], mode="csr", sparsity_arrays=spa,
                           nthreads=1, fast=True)
        times.append(time.perf_counter() - t0)
    return el.shape[0] / min(times) / 1e6


def run_reference(args):
    """The reference algorithm's CPU implementation (the C restatement of _GlobalAssemblyDF_,
    liboracle_fast.so, compiled with the reference's optimisation flags) on all host threads:
    each step one full assembly of the workload. Also the one-thread rate on a sample."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle
    W = workload(args.workload)
    spa = oracle.sparsity(W["elements"], W["points"].shape[0])
    nthreads = oracle.max_threads()
    nelem = W["elements"].shape[0]
    for _ in range(args.warmup):
        oracle.assemble_df(W["material"], W["params"], W["points"], W["elements"], W["x"], W["Jm"], W["w"],
                           mode="csr", sparsity_arrays=spa, nthreads=nthreads, fast=True)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.assemble_df(W["material"], W["params"], W["points"], W["elements"], W["x"], W["Jm"], W["w"],
                           mode="csr", sparsity_arrays=spa, nthreads=nthreads, fast=True)
    dt = time.perf_counter() - t0
    value = nelem * args.steps / dt / 1e6
    v1 = one_core_rate(W)
    line = dict(metric="FP64 assembly throughput (tangent CSR + residual)", value=value, unit="Melem/s",
                n_gpus=args.gpus, steps=args.steps, warmup=args.warmup, ms_per_step=dt / args.steps * 1e3,
                higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f64", data="synthetic",
                config=bench_config(W, spa[0].shape[0], int(os.environ.get("WORLD_SIZE", "1"))),
                impl="reference",
                cpu_baseline=dict(value=value, unit="Melem/s", cores=nthreads, kind="port", cpu_model=cpu_model(),
                                  host_threads=os.cpu_count(), value_1core=v1,
                                  sample="%d steps, each a full assembly of all %d elements on %d threads; one-thread "
                                         "rate on the first 6000 elements" % (args.steps, nelem, nthreads)),
                e2e=dict(value=value, unit="Melem/s", h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line), flush=True)


def cpu_baseline_subprocess(args, steps=20):
    """The reference arm run as its own process (`--impl reference`), so that the CPU figure this
    arm reports comes from the same code, the same kind of process and the same threads as the
    reference arm's line; returns its cpu_baseline object."""
    cmd = [sys.executable, os.path.abspath(__file__), "--impl", "reference", "--steps", str(steps), "--warmup", "3",
           "--workload", args.workload]
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=900)
    for line in r.stdout.splitlines()[::-1]:
        if line.startswith("{"):
            cb = json.loads(line)["cpu_baseline"]
            cb["sample"] = "reference arm run as a subprocess: " + cb["sample"]
            return cb
    raise RuntimeError("CPU baseline subprocess failed: " + r.stderr[-2000:])


def parity_check(W, asm, V, T):
    """The bench's own last-step outputs against the oracle (IEEE build, all host threads), outside
    the timed region: the device CSR pattern and element-to-nonzero maps bit-exact against the
    oracle's, V and T in relative Frobenius norm."""
    from oracle import oracle
    ind, ptr, dl, dg = oracle.sparsity(W["elements"], W["points"].shape[0])
    exact = (np.array_equal(ind, asm.indices.cpu().numpy()) and np.array_equal(ptr, asm.indptr.cpu().numpy())
             and np.array_equal(dl, asm.data_local.cpu().numpy()) and np.array_equal(dg, asm.data_global.cpu().numpy()))
    Vo, To = oracle.assemble_df(W["material"], W["params"], W["points"], W["elements"], W["x"], W["Jm"], W["w"],
                                mode="csr", sparsity_arrays=(ind, ptr, dl, dg), nthreads=oracle.max_threads())
    Vf, Tf = oracle.assemble_df(W["material"], W["params"], W["points"], W["elements"], W["x"], W["Jm"], W["w"],
                                mode="csr", sparsity_arrays=(ind, ptr, dl, dg), nthreads=oracle.max_threads(),
                                fast=True)
    Vd, Td = V.double().cpu().numpy(), T.cpu().numpy()
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))  # noqa: E731
    return dict(K=rel(Vd, Vo), T=rel(Td, To), pattern_bit_exact=bool(exact),
                fp64_spread=dict(K=rel(Vf, Vo), T=rel(Tf, To),
                                 note="the same reference algorithm in FP64 with reassociation and contraction "
                                      "(-ffast-math build) against its IEEE build: the rounding sensitivity of this "
                                      "mesh (sliver tetrahedra), the floor no FP64 evaluation order goes below"),
                checker="oracle (C restatement of _GlobalAssemblyDF_, IEEE build), full workload")


# ------------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------------
def run_ours(args):
    import torch
    import torch.distributed as dist
    import florence_gb300 as fl

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    W = workload(args.workload)
    nelem, npe = W["elements"].shape
    nq = int(np.ravel(W["w"]).shape[0])
    nnode = W["points"].shape[0]
    asm = fl.DeviceAssembler(W["points"], W["elements"], W["Jm"], W["w"], W["material"], W["params"], mode="csr",
                             device=dev)
    x = torch.from_numpy(W["x"]).to(dev)
    mixed = args.arith == "mixed"
    V = torch.zeros(asm.nnz, dtype=torch.float32 if mixed else torch.float64, device=dev)
    T = torch.zeros(nnode * 3, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step(ev=None):
        V.zero_()
        T.zero_()
        if ev is not None:
            ev[0].record(stream)
        if mixed:
            asm.assemble_mixed(x, V32=V, T=T)
        else:
            asm.assemble(x, V=V, T=T)
        if ev is not None:
            ev[1].record(stream)

    fl.set_arithmetic("fp64" if mixed else args.arith)
    fl.set_tensor_core_tiling(*[int(v) for v in args.tc_tiling.split(",")])
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    asm.check_flags("bench warm-up")
    fp64_peak = fl.fp64_peak_gflops() / 1e3  # TFLOP/s, measured in this run
    fp32_peak = fl.fp32_peak_gflops() / 1e3
    kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0.record(stream)
        for k in range(args.steps):
            step(kev[k])
        t1.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    from florence_gb300.replicas import job_throughput
    rate, ms, _ = job_throughput(nelem * args.steps, t0.elapsed_time(t1), device=dev)
    kernel_ms = float(np.mean([a.elapsed_time(b) for a, b in kev]))
    clocks = clk.summary()
    value = rate / 1e6

    # roofline of the dominant kernel (assemble_df_kernel): FP64-pipe bound
    f_alg = flops_alg(npe, nq, W["material"]) * nelem
    f_exe = flops_executed(npe, nq, W["material"]) * nelem
    achieved = f_alg / (kernel_ms * 1e-3) / 1e12
    bmin = bytes_min(nnode, nelem, npe, asm.nnz)
    hbm_peak = json.load(open(PEAKS))["hbm_gbs"] if os.path.exists(PEAKS) else 6800.0
    if args.arith == "fp64":
        roofline = dict(bound="fp64", achieved=achieved, peak=fp64_peak, unit="TFLOP/s", frac=achieved / fp64_peak,
                        peak_source="FP64 FMA microkernel measured in this run (no FP64 figure in "
                                    "MEASURED_PEAKS.json)",
                        executed_frac=f_exe / (kernel_ms * 1e-3) / 1e12 / fp64_peak)
    elif mixed:  # split-BF16 tangent: six BF16 MMA products per element contraction
        npad = (npe + 15) // 16 * 16           # MMA N: nodes padded to 16
        mpad = (9 * npe + 127) // 128 * 128    # MMA M: 128-row tiles
        kpad = (3 * nq + 15) // 16 * 16        # K steps of 16
        tflop = 6 * 2.0 * mpad * npad * kpad * nelem / (kernel_ms * 1e-3) / 1e12
        peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}
        bf16_peak = peaks.get("bf16_tflops", 1900.0)
        roofline = dict(bound="tensor", achieved=tflop, peak=bf16_peak, unit="TFLOP/s", frac=tflop / bf16_peak,
                        peak_source="MEASURED_PEAKS.json bf16_tflops" if "bf16_tflops" in peaks else "fallback",
                        note="the tensor work per element is small; the FP64 Gauss-point kernel and the scatter "
                             "bound the step", fp64_equivalent_tflops=achieved)
    elif args.arith == "tensor":  # FP64 tangent on the tensor cores: 21 digit-pair products per K step
        npad = (npe + 15) // 16 * 16
        mpad = (9 * npe + 127) // 128 * 128
        kpad = (3 * nq + 15) // 16 * 16
        tflop = 21 * 2.0 * mpad * npad * kpad * nelem / (kernel_ms * 1e-3) / 1e12
        peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}
        bf16_peak = peaks.get("bf16_tflops", 1900.0)
        roofline = dict(bound="tensor", achieved=tflop, peak=bf16_peak, unit="TFLOP/s", frac=tflop / bf16_peak,
                        peak_source="MEASURED_PEAKS.json bf16_tflops" if "bf16_tflops" in peaks else "fallback",
                        note="BF16 digit products; the operand build and the scatter bound the step",
                        fp64_equivalent_tflops=achieved, fp64_equivalent_frac=achieved / fp64_peak)
    elif args.arith == "reference_tensor":  # tiles of 14 elements x 80 node pairs, 28 BF16 plane products
        pairs = npe * (npe + 1) // 2
        nch = (pairs + 79) // 80
        nks = (9 * nq + 15) // 16
        ntiles = (nelem + 13) // 14
        tflop = 28 * 2.0 * 128 * 80 * 16 * nks * nch * ntiles / (kernel_ms * 1e-3) / 1e12
        peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}
        bf16_peak = peaks.get("bf16_tflops", 1900.0)
        roofline = dict(bound="tensor", achieved=tflop, peak=bf16_peak, unit="TFLOP/s", frac=tflop / bf16_peak,
                        peak_source="MEASURED_PEAKS.json bf16_tflops" if "bf16_tflops" in peaks else "fallback",
                        note="BF16 digit-plane products of the whole assembly call (Gauss-point kernel included "
                             "in the time)", fp64_equivalent_tflops=achieved,
                        fp64_equivalent_frac=achieved / fp64_peak)
    else:  # the contraction runs as float pairs on the FP32 pipe
        instr = 12.0 * pair_macs(npe, nq) * nelem
        ach_i = instr / (kernel_ms * 1e-3) / 1e12
        roofline = dict(bound="fp32", achieved=ach_i, peak=fp32_peak / 2, unit="T FP32-pipe instr/s",
                        frac=ach_i / (fp32_peak / 2),
                        peak_source="FP32 FMA microkernel measured in this run (instructions/s = FLOP/s / 2)",
                        fp64_equivalent_tflops=achieved, fp64_equivalent_frac=achieved / fp64_peak,
                        instr_per_launch=instr)
    tag = {"fp64": "assemble_df_%s_%s", "float_pair": "contract_float_pair_%s_%s", "tensor": "contract_oz_%s_%s",
           "reference_tensor": "rt_contract_%s_%s", "mixed": "contract_tc_%s_%s"}[args.arith] % (
        W["desc"]["element"], W["desc"]["material"])
    roofline.update(traffic=traffic_from_profile(tag), flop_alg_per_launch=f_alg, flop_executed_per_launch=f_exe,
                    kernel_ms=kernel_ms,
                    hbm=dict(bytes_min_per_launch=bmin, achieved_gbs=bmin / (kernel_ms * 1e-3) / 1e9,
                             peak_gbs=hbm_peak, frac=bmin / (kernel_ms * 1e-3) / 1e9 / hbm_peak,
                             peak_source="MEASURED_PEAKS.json" if os.path.exists(PEAKS) else "fallback 6.8 TB/s"))

    # the same assembly scattering by row search (the drop-in's CSR path), device time
    squeeze = None
    if rank == 0 and not mixed and not args.no_e2e:
        sq = fl.DeviceAssembler(W["points"], W["elements"], W["Jm"], W["w"], W["material"], W["params"],
                                mode="squeeze", device=dev, sparsity=(asm.indices, asm.indptr, None, None))
        Vs = torch.zeros_like(V)
        for _ in range(3):
            Vs.zero_()
            sq.assemble(x, V=Vs, T=T.zero_())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        nsq = max(3, min(args.steps, 10))
        for _ in range(nsq):
            Vs.zero_()
            T.zero_()
            sq.assemble(x, V=Vs, T=T)
        e1.record(stream)
        torch.cuda.synchronize()
        ms_sq = e0.elapsed_time(e1) / nsq
        squeeze = dict(ms_per_step=ms_sq, value=nelem / (ms_sq * 1e-3) / 1e6, unit="Melem/s",
                       note="CSR positions found by row search in the pattern (no element-to-nonzero maps): "
                            "the scatter of the drop-in callable")
        del sq
        # the deterministic mode: node-disjoint colours assembled one after another
        dt = fl.DeviceAssembler(W["points"], W["elements"], W["Jm"], W["w"], W["material"], W["params"],
                                mode="squeeze", device=dev, sparsity=(asm.indices, asm.indptr, None, None),
                                deterministic=True)
        for _ in range(3):
            Vs.zero_()
            dt.assemble(x, V=Vs, T=T.zero_())
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(nsq):
            Vs.zero_()
            T.zero_()
            dt.assemble(x, V=Vs, T=T)
        e1.record(stream)
        torch.cuda.synchronize()
        ms_dt = e0.elapsed_time(e1) / nsq
        squeeze["deterministic"] = dict(ms_per_step=ms_dt, value=nelem / (ms_dt * 1e-3) / 1e6, unit="Melem/s",
                                        colours=len(dt._colour),
                                        note="bit-reproducible: node-disjoint element colours assembled in turn")
        del dt, Vs

    # parity of the timed workload against the oracle (outside the timed region): rerun one step
    parity = None
    if rank == 0 and not args.no_parity:
        step()
        torch.cuda.synchronize()
        parity = parity_check(W, asm, V, T)

    # end to end through the drop-in callable (host numpy in and out, copies inside)
    e2e = None
    if rank == 0 and not args.no_e2e and not mixed:  # the drop-in returns the FP64 tangent
        e2e = e2e_dropin(W, asm, args)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline_subprocess(args)

    if rank == 0:
        line = dict(metric="FP64 assembly throughput (tangent CSR + residual)" if not mixed else
                    "split-BF16 tangent assembly throughput (FP32 CSR values + FP64 residual)",
                    value=value, unit="Melem/s", arithmetic=args.arith,
                    n_gpus=world, steps=args.steps, warmup=args.warmup, ms_per_step=ms / args.steps,
                    higher_is_better=True, scaling="weak", vs_baseline=None,
                    dtype={"fp64": "f64", "float_pair": "f64 (float-pair contraction)",
                           "reference_tensor": "f64 (seven-digit BF16 plane products on tcgen05, exact levels, "
                                               "integer recombination)",
                           "tensor": "f64 (six-digit BF16 products, exact f32 levels, float-pair recombination)",
                           "mixed": "bf16x3 products, f32 accumulate; f64 residual"}[args.arith], data="synthetic",
                    config=bench_config(W, asm.nnz, world),
                    roofline=roofline, cpu_baseline=cpu, e2e=e2e, clocks=clocks, parity=parity, squeeze=squeeze,
                    gpu_launches=args.steps * (mixed_launches(nelem, nq) if mixed else
                                               tensor_launches(nelem, nq) if args.arith == "tensor" else
                                               rt_launches(nelem, nq) if args.arith == "reference_tensor" else
                                               assembly_launches(nelem, npe, nq)))
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_newton(args):
    """Newton load stepping of the tet p=3 beam (x=0 clamped, uniform downward traction 0.01 on
    x=4, 10 increments, relative residual 1e-10), FP64 tangent, device block-Jacobi PCG."""
    import torch
    import florence_gb300 as fl
    from florence_gb300.newton import NewtonSolver, build_beam_problem
    cells = (48, 12, 12) if args.workload != "beam_s" else (24, 6, 6)
    P, el, Jm, w, fixed, f = build_beam_problem(*cells, traction=0.01)
    asm = fl.DeviceAssembler(P, el, Jm, w, "MooneyRivlin", (0.5, 0.5, 20.0), mode="csr")
    from florence_gb300 import meshes
    g = np.load(os.path.join(GOLDEN, "tet_p3_mr_jitter.npz"))
    pat = meshes.local_pattern(g["points"], g["elements"], 0, "tet")
    tangents = {"both": ["fp64", "mixed"], "all": ["fp64", "mixed", "hybrid"]}.get(args.tangent, [args.tangent])
    runs = {}
    linear = args.linear if args.tangent == "fp64" else "pcg"  # the p-multigrid cycle takes the FP64 tangent
    lin = dict(linear=linear, pattern=pat if linear == "pmg" else None)
    for tg in tangents:
        # warm-up: module loading, one assembly and one short linear solve
        NewtonSolver(asm, fixed, f, n_increments=1, max_iter=1, pcg_maxiter=32, tangent=tg, spmv=args.spmv,
                     **lin).solve()
        runs[tg] = NewtonSolver(asm, fixed, f, n_increments=10, tol=1e-10, tangent=tg, spmv=args.spmv,
                                max_iter=args.newton_max_iter, forcing=args.forcing, **lin).solve()
    out = runs[tangents[-1]]
    extra = {}
    if len(runs) > 1:
        a = runs["fp64"]
        for tg, b in runs.items():
            extra[tg] = dict(wall_s=b["wall_s"], newton_iters=b["newton_iters"], pcg_iters=b["pcg_iters"],
                             failed=b["failed"])
            if tg != "fp64":
                extra[tg]["rel_l2_vs_fp64"] = float(torch.linalg.vector_norm(b["u"] - a["u"]) /
                                                    torch.linalg.vector_norm(a["u"]))
    u = out["u"].cpu().numpy().reshape(-1, 3)
    tip = np.abs(P[:, 0] - 4.0) < 1e-9
    incs = [dict(increment=i["increment"], newton=i["newton_iters"],
                 pcg=[h["pcg_iters"] for h in i["history"]], rel=[h["rel"] for h in i["history"]])
            for i in out["increments"]]
    line = dict(metric=("Newton wall time to rel-res 1e-10 (10 load increments, %s tangent, "
                        + ("flexible CG with the p-multigrid cycle)" if linear == "pmg" else "block-Jacobi PCG)"))
                       % {"fp64": "FP64", "mixed": "split-BF16 tensor-core FP32",
                          "hybrid": "split-BF16 FP32 far from the solution, FP64 near it",
                          "both": "split-BF16 tensor-core FP32 (FP64 run alongside)",
                          "all": "hybrid split-BF16/FP64 (FP64 and split-BF16 runs alongside)"}[args.tangent],
                value=out["wall_s"], unit="s", n_gpus=1, steps=1, warmup=1, higher_is_better=False,
                scaling="weak", vs_baseline=None, dtype="f64", data="synthetic", tangent=args.tangent,
                spmv=args.spmv if args.tangent != "mixed" else "fp32 values, float-pair product",
                forcing=args.forcing, linear=linear, pcg_loop=args.pcg_loop,
                config=dict(workload="tet p=3 beam 4x1x1 (%dx%dx%d jittered lattice), Mooney-Rivlin mu1=mu2=0.5 "
                                     "lambda=20, x=0 clamped, traction (0,0,-0.01) on x=4" % cells,
                            nelem=int(el.shape[0]), nnode=int(P.shape[0]), nnz=int(asm.nnz)),
                newton_iters=out["newton_iters"], pcg_iters=out["pcg_iters"], failed=out["failed"],
                tip_uz=float(u[tip, 2].mean()), increments=incs,
                **{k: out[k] for k in ("mg_cycles", "mg_coarse_iters") if k in out}, **extra)
    print(json.dumps(line), flush=True)


def run_pcg(args):
    """Block-Jacobi PCG iterations on the FP64 tangent of the tet p=3 beam (the Newton
    configuration's matrix at the unloaded state, 95 M nonzeros), a fixed count of iterations
    (no convergence stop), per product mode: float-pair split values on the FP32 pipe (Newton's
    default) and FP64 products. Reports the time per iteration and the achieved bandwidth by
    algorithmic bytes against the measured HBM peak."""
    import torch
    import florence_gb300 as fl
    from florence_gb300.newton import build_beam_problem, pcg, pcg_workspace
    cells = (48, 12, 12) if args.workload != "beam_s" else (24, 6, 6)
    P, el, Jm, w, fixed, f = build_beam_problem(*cells, traction=0.01)
    asm = fl.DeviceAssembler(P, el, Jm, w, "MooneyRivlin", (0.5, 0.5, 20.0), mode="csr")
    V, _ = asm.assemble(torch.from_numpy(P).cuda())
    fx = torch.from_numpy(fixed.astype(np.int8)).cuda()
    b = torch.from_numpy(np.where(fixed, 0.0, f)).cuda()
    n, nnz = asm.nnode * 3, asm.nnz
    # algorithmic bytes per iteration: values (8 B per nonzero either way: FP64, or the hi + lo
    # float pair), one column index per 3x3 block, the row pointers, and the vector streams of
    # the three kernels (K1 reads p and writes q as float pairs, 16 B per dof; K2 reads x, p, q, r
    # and the 3x3 block inverse, 64 B, and writes x, r, z, 24 B; K3 reads z, p and writes p and
    # its float pair, 32 B)
    nbytes = 8 * nnz + 4 * (nnz // 9) + 4 * (n + 1) + 136 * n
    peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    res = {}
    for spmv in ("split", "fp64"):
        ws = pcg_workspace(asm, V, spmv)
        pcg(asm, V, b, fx, rtol=1e-30, maxiter=args.warmup * 16, workspace=ws, spmv=spmv)  # lanes autotune
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(0) as clk:
            e0.record()
            _, it, rel = pcg(asm, V, b, fx, rtol=1e-30, maxiter=args.pcg_iters, workspace=ws, spmv=spmv)
            e1.record()
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / it
        res[spmv] = dict(ms_per_iter=ms, iterations=it, achieved_gbs=nbytes / (ms * 1e-3) / 1e9,
                         frac=nbytes / (ms * 1e-3) / 1e9 / hbm, clocks=clk.summary())
    line = dict(metric="block-Jacobi PCG time per iteration (float-pair split SpMV)", value=res["split"]["ms_per_iter"],
                unit="ms", n_gpus=1, steps=args.pcg_iters, warmup=args.warmup * 16, higher_is_better=False,
                scaling="weak", vs_baseline=None, dtype="f64", data="synthetic",
                config=dict(workload="tet p=3 beam 4x1x1 (%dx%dx%d jittered lattice), Mooney-Rivlin FP64 tangent at "
                                     "the unloaded state, x=0 clamped" % cells, n=n, nnz=nnz,
                            inputs="larger than L2 (values %.0f MB)" % (8 * nnz / 1e6)),
                roofline=dict(bound="hbm", achieved=res["split"]["achieved_gbs"], peak=hbm, unit="GB/s",
                              frac=res["split"]["frac"], bytes_per_iter=nbytes,
                              peak_source="MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback"),
                split=res["split"], fp64=res["fp64"], clocks=res["split"]["clocks"], pcg_loop=args.pcg_loop)
    print(json.dumps(line), flush=True)


def run_explicit(args):
    """Explicit dynamics of the p=2 hex beam (64x8x8 elements on [0,8]x[0,1]x[0,1], both ends
    clamped, neo-Hookean mu=1 lambda=1000 rho=1, lumped mass, v_z = 0.1 sin(pi x / L) at t=0,
    dt = 0.9 x critical, 10 000 central-difference steps), internal force in FP64 and in FP32."""
    import torch
    from florence_gb300.explicit import ExplicitSolver, build_explicit_beam
    n = (64, 8, 8) if args.workload != "beam_s" else (32, 4, 4)
    nsteps = args.explicit_steps
    P, el, Jm, w, B, fixed = build_explicit_beam(*n, L=8.0)
    s = ExplicitSolver(P, el, Jm, w, B, 1.0, 1000.0, 1.0, fixed)
    dtc, lam = s.critical_dt(iters=30)
    dt = 0.9 * dtc
    v0 = np.zeros_like(P)
    v0[:, 2] = 0.1 * np.sin(np.pi * P[:, 0] / 8.0)
    res = {}
    for mode in ("fp64", "pair", "fp32"):
        s.run(v0.ravel(), dt, 200, mode=mode, energy_every=0)   # warm-up (graph capture, clocks)
        r = s.run(v0.ravel(), dt, nsteps, mode=mode, energy_every=max(1, nsteps // 50))
        E = np.array([k + i for _, k, i in r["energy"]])
        res[mode] = dict(wall_s=r["wall_s"], steps=r["steps"], steps_per_s=r["steps"] / r["wall_s"],
                         energy_drift_max=float(np.abs(E / E[0] - 1.0).max()),
                         energy_drift_final=float(E[-1] / E[0] - 1.0), blowup=r["blowup"], u=r["u"])
    l2 = float(torch.linalg.vector_norm(res["fp32"]["u"] - res["fp64"]["u"]) /
               torch.linalg.vector_norm(res["fp64"]["u"]))
    l2p = float(torch.linalg.vector_norm(res["pair"]["u"] - res["fp64"]["u"]) /
                torch.linalg.vector_norm(res["fp64"]["u"]))
    for m in res:
        res[m].pop("u")
    line = dict(metric="explicit central-difference steps per second (FP64-accurate internal force: float-pair "
                       "arithmetic, trajectory within l2_pair_vs_fp64 of the FP64 kernel)",
                value=res["pair"]["steps_per_s"], unit="steps/s", n_gpus=1, steps=nsteps, warmup=200,
                higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f64", data="synthetic",
                config=dict(workload="p=2 hex beam %dx%dx%d on [0,8]x[0,1]x[0,1], ends clamped, neo-Hookean mu=1 "
                                     "lambda=1000 rho=1, lumped mass, v_z=0.1 sin(pi x/8)" % n,
                            nelem=int(el.shape[0]), nnode=int(P.shape[0]), gauss_points=int(np.ravel(w).shape[0]),
                            dt=dt, dt_critical=dtc, omega_max=float(np.sqrt(lam))),
                fp64=res["fp64"], pair=res["pair"], fp32=res["fp32"], l2_fp32_vs_fp64=l2, l2_pair_vs_fp64=l2p)
    print(json.dumps(line), flush=True)


def run_batched(args):
    """512 independent cube meshes (n^3 hexes, n ~ U{2..12}, p ~ U{1..4}, per-instance neo-Hookean
    parameters, displacement U(-0.01, 0.01)): FP64 tangent + residual of all instances, one
    launch pair per element order and sub-batch (sub-batches keep CSR values and indices under a
    memory budget and below 2^31 nonzeros), Gauss-point chunk autotuned per order; then the
    split-BF16 variant."""
    import torch
    from florence_gb300.batched import BatchedAssembler, build_instance, config4_instances, hex_tables
    specs = config4_instances(args.instances, seed=2)
    budget = args.batch_gb * 1e9
    npe_of = {1: 8, 2: 27, 3: 64, 4: 125}
    nnz_per_elem = {1: 243, 2: 4608, 3: 30375, 4: 124416}   # asymptotic, for grouping only
    totals = dict(elements=0, nnz=0, fp64_ms=0.0, mixed_ms=0.0, setup_s=0.0)
    per_p = {}
    for p in (1, 2, 3, 4):
        pat, Jm, w = hex_tables(p)
        group, gbytes, groups = [], 0.0, []
        nnz_cap = 1.8e9          # int32 CSR positions: a sub-batch stays below 2^31 nonzeros
        for sp in [s_ for s_ in specs if s_["p"] == p]:
            b = sp["n"] ** 3 * nnz_per_elem[p] * 16.0
            if group and (gbytes + b > budget or (gbytes + b) / 16.0 > nnz_cap):
                groups.append(group)
                group, gbytes = [], 0.0
            group.append(sp)
            gbytes += b
        if group:
            groups.append(group)
        tuned = None
        pe = dict(instances=0, elements=0, nnz=0, fp64_ms=0.0, mixed_ms=0.0, sub_batches=len(groups))
        for gi, grp in enumerate(groups):
            t0 = time.perf_counter()
            B = BatchedAssembler([build_instance(sp, pat) for sp in grp], Jm, w, "NeoHookean", maps=False)
            torch.cuda.synchronize()
            totals["setup_s"] += time.perf_counter() - t0
            if tuned is None:
                tuned = B.autotune()
            V = torch.zeros(B.nnz, dtype=torch.float64, device="cuda")
            T = torch.zeros(B.nnode * 3, dtype=torch.float64, device="cuda")
            for mixed in (False, True):
                Vm = torch.zeros(B.nnz, dtype=torch.float32, device="cuda") if mixed else V
                B.assemble(Vm, T, mixed=mixed)  # warm-up
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                Vm.zero_()
                T.zero_()
                torch.cuda.synchronize()
                e0.record()
                B.assemble(Vm, T, mixed=mixed)
                e1.record()
                torch.cuda.synchronize()
                pe["mixed_ms" if mixed else "fp64_ms"] += e0.elapsed_time(e1)
                del Vm
            if int(B.flags.item()) & 2:
                raise RuntimeError("batched assembly reported out-of-range indices")
            pe["instances"] += len(grp)
            pe["elements"] += B.nelem
            pe["nnz"] += B.nnz
            del B, V, T
            torch.cuda.empty_cache()
        pe["autotune"] = tuned
        per_p[p] = pe
        for k in ("elements", "nnz", "fp64_ms", "mixed_ms"):
            totals[k] += pe[k]
    value = totals["elements"] / (totals["fp64_ms"] * 1e-3) / 1e6
    line = dict(metric="batched FP64 assembly throughput (tangent CSR + residual, uneven instances)", value=value,
                unit="Melem/s", n_gpus=1, steps=1, warmup=1, higher_is_better=True, scaling="weak",
                vs_baseline=None, dtype="f64", data="synthetic",
                config=dict(workload="%d independent hex cubes, n~U{2..12}, p~U{1..4}, neo-Hookean mu~U(0.5,2) "
                                     "lambda~U(5,50), u~U(-0.01,0.01), default_rng(2)" % args.instances,
                            elements=int(totals["elements"]), nnz=int(totals["nnz"]),
                            sub_batch_budget_gb=args.batch_gb),
                fp64_ms=totals["fp64_ms"], mixed_ms=totals["mixed_ms"],
                mixed_melem_s=totals["elements"] / (totals["mixed_ms"] * 1e-3) / 1e6,
                setup_s=totals["setup_s"], per_order=per_p)
    print(json.dumps(line), flush=True)


def e2e_dropin(W, asm, args):
    """The reference-facing call (_LowLevelAssemblyDF__<Mat>_) with host arrays, as Florence's
    Newton loop makes it: the first calls upload the mesh, its tables and the CSR pattern (kept on
    the device between calls with the same arrays); every timed call uploads the coordinates
    Eulerx, assembles, and downloads V and T into host arrays."""
    import torch
    import florence_gb300 as fl
    spa = (asm.indices.cpu().numpy(), asm.indptr.cpu().numpy(), asm.data_local.cpu().numpy(),
           asm.data_global.cpu().numpy())
    mat = W["material"]
    p = W["params"]
    material = types.SimpleNamespace(H_VoigtSize=6, is_transversely_isotropic=False, rho=1.0, mtype=mat)
    if mat == "NeoHookean":
        material.mu, material.lamb = p[0], p[1]
    else:
        material.mu1, material.mu2, material.lamb = p
    fs = types.SimpleNamespace(Jm=W["Jm"], AllGauss=np.ravel(W["w"])[:, None])
    form = types.SimpleNamespace(ndim=3, nvar=3, fields="mechanics")
    mesh = types.SimpleNamespace(points=W["points"], elements=W["elements"].astype(np.uint64),
                                 nelem=W["elements"].shape[0])
    solver = types.SimpleNamespace(requires_geometry_update=1, recompute_sparsity_pattern=False,
                                   squeeze_sparsity_pattern=False, indices=spa[0], indptr=spa[1],
                                   data_local_indices=spa[2], data_global_indices=spa[3])
    fn = getattr(fl, "_LowLevelAssemblyDF__" + mat + "_")
    Ep = np.zeros(W["points"].shape[0])
    V = T = None
    for _ in range(3):  # as in the timed loop, each call runs while the previous result is held
        V, T = fn(solver, fs, form, mesh, material, W["x"], Ep)
    steps = max(3, min(args.steps, 10))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        V, T = fn(solver, fs, form, mesh, material, W["x"], Ep)
    dt = (time.perf_counter() - t0) / steps
    # uploaded per timed call: the coordinates (the mesh, tables and pattern stay on the device)
    h2d = W["x"].nbytes
    d2h = V.nbytes + T.nbytes
    return dict(value=W["elements"].shape[0] / dt / 1e6, unit="Melem/s", h2d_bytes_per_step=int(h2d),
                d2h_bytes_per_step=int(d2h), ms_per_step=dt * 1e3, steps=steps,
                path="florence_gb300._LowLevelAssemblyDF__%s_ (host numpy in; outputs in pooled pinned host "
                     "buffers; mesh kept on the device between calls)" % mat)


def run_warmstart(args):
    """Learned warm start on the p=2 tet plate (about 20k tets, [0,2]x[0,1]x[0,0.2], x=0 clamped,
    in-plane traction on x=2, neo-Hookean): training solves over sampled (mu, lambda/mu,
    traction), a 64-mode POD basis of their converged increments, the network trained on the GPU,
    then held-out solves from the previous-increment guess and from the network's guess."""
    import torch
    from florence_gb300 import warmstart as W
    t0 = time.perf_counter()
    prob = W.build_plate_problem()
    solver = W.PlateSolver(prob, n_increments=args.ws_increments, tol=1e-10)
    solver.solve(1.0, 10.0, 0.1)                          # warm-up: module loading, first assembly
    train = W.sample_parameters(args.ws_train, seed=3)
    test = W.sample_parameters(args.ws_test, seed=4)
    t1 = time.perf_counter()
    X, U, stats = W.generate_snapshots(solver, train)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    ws, hist, sv, proj = W.train_warm_start(X, U, modes=64, steps=args.ws_steps)
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    hybrid = W.PlateSolver(prob, n_increments=args.ws_increments, tol=1e-10, tangent="hybrid")
    hybrid.solve(1.0, 10.0, 0.1)                          # warm-up of the mixed kernels
    rows, tot = W.evaluate_warm_start(solver, ws, test, {"warm": solver, "mixed_warm": hybrid})
    t4 = time.perf_counter()
    line = dict(metric="Newton wall time to rel-res 1e-10 over the held-out solves: split-BF16/FP64 hybrid "
                       "tangent with the network warm start (plain FP64 Newton alongside)",
                value=tot["mixed_warm"]["wall_s"], unit="s", n_gpus=1, steps=len(test), warmup=1,
                higher_is_better=False, scaling="weak", vs_baseline=None, dtype="f64", data="synthetic",
                config=dict(workload="p=2 tet plate 2x1x0.2 (38x19x4 jittered lattice), neo-Hookean mu~U(0.5,2) "
                                     "lambda/mu~U(2,100), traction~U(0,0.5) (+x) on x=2, x=0 clamped, "
                                     "%d increments, |R| <= 1e-10 |F|" % args.ws_increments,
                            nelem=int(prob[1].shape[0]), nnode=int(prob[0].shape[0]), train_solves=len(train),
                            test_solves=len(test), snapshots=int(U.shape[1]), pod_modes=64,
                            network="3-256-256-64 GELU, BF16 operands, FP32 master, Adam"),
                plain=tot["plain"], warm=tot["warm"], mixed_warm=tot["mixed_warm"], increments=tot["increments"],
                newton_ratio=tot["warm"]["newton"] / max(1, tot["plain"]["newton"]),
                wall_ratio_warm=tot["warm"]["wall_s"] / max(1e-12, tot["plain"]["wall_s"]),
                wall_ratio_mixed_warm=tot["mixed_warm"]["wall_s"] / max(1e-12, tot["plain"]["wall_s"]),
                max_solution_diff=max(tot["warm"]["max_du"], tot["mixed_warm"]["max_du"]),
                training=dict(failed=sum(s_["failed"] for s_ in stats), generate_s=t2 - t1, train_s=t3 - t2,
                              evaluate_s=t4 - t3, loss_first=hist[0], loss_last=hist[-1], pod_projection_err=proj,
                              sv_ratio_64=float(sv[-1] / sv[0])))
    print(json.dumps(line), flush=True)


def run_meshing(args):
    """High-order tet mesh generation on the device (fl_RaiseTetOrder): a box of Kuhn-split cubes
    (10.6 M linear tets, 1.8 M vertices) raised to p=3 with the equispaced 20-node layout. One
    step = one call with preallocated outputs (counting, entity numbering, node numbers and
    positions, two host synchronisations). value = linear tets per second; e2e = the same call from host
    numpy arrays with the mesh copied back; cpu_baseline = the host builder (numpy, one thread)
    on a 24 x 24 x 24 box."""
    import itertools
    import torch
    from florence_gb300 import meshes
    cells = (192, 96, 96) if args.workload != "beam_s" else (48, 24, 24)
    rows = sorted((c for c in itertools.product(range(4), repeat=4) if sum(c) == 3),
                  key=lambda c: (-max(c), [-x for x in c]))
    lam = np.array(rows, np.float64) / 3.0
    P, el = meshes.kuhn_tet_box(cells, (2.0, 1.0, 1.0))
    nelem, nvert = el.shape[0], P.shape[0]
    Pd, eld = torch.from_numpy(P).cuda(), torch.from_numpy(el).cuda()
    X3, E3 = meshes.raise_tet_order_device(Pd, eld, lam)
    nnode = X3.shape[0]
    out_p, out_e = torch.empty((nnode, 3), dtype=torch.float64, device="cuda"), E3
    del X3
    for _ in range(args.warmup):
        meshes.raise_tet_order_device(Pd, eld, lam, out_points=out_p, out_elements=out_e)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = max(1, args.steps)
    with ClockSampler(0) as clk:
        e0.record()
        for _ in range(steps):
            meshes.raise_tet_order_device(Pd, eld, lam, out_points=out_p, out_elements=out_e)
        e1.record()
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    value = nelem / (ms * 1e-3) / 1e6
    # compulsory bytes: linear tets and vertices read once, the high-order mesh written once
    npe = lam.shape[0]
    nbytes = 32 * nelem + 24 * nvert + 8 * npe * nelem + 24 * nnode
    peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    # end to end: host arrays in, host mesh out
    e2e = None
    if not args.no_e2e:
        t_h = []
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            Xh, Eh = meshes.raise_tet_order_device(P, el, lam)
            Xh, Eh = Xh.cpu().numpy(), Eh.cpu().numpy()
            t_h.append(time.perf_counter() - t0)
        e2e = dict(value=nelem / min(t_h[1:]) / 1e6, unit="Melem/s", h2d_bytes_per_step=P.nbytes + el.nbytes,
                   d2h_bytes_per_step=Xh.nbytes + Eh.nbytes)
    cpu = None
    if not args.no_cpu:
        Ps, els = meshes.kuhn_tet_box((24, 24, 24), (2.0, 1.0, 1.0))
        t0 = time.perf_counter()
        meshes.raise_tet_order(Ps, els, lam)
        dt = time.perf_counter() - t0
        cpu = dict(value=els.shape[0] / dt / 1e6, unit="Melem/s", cores=1, kind="port",
                   sample="host builder (numpy np.unique of entity keys) on a 24x24x24 Kuhn box, %d tets" % els.shape[0])
    launches = 18  # count, degree, fill, entities (count and write), nodes, four 3-kernel scans
    # hexes (fl_RaiseHexOrder): a structured box of linear hexes raised to p=3 with the reference's
    # 64-node Gauss-Lobatto layout (taken from a golden fixture)
    g = np.load(os.path.join(GOLDEN, "hex_p3_nh.npz"))
    xi = meshes.local_pattern(g["points"], g["elements"], 0, "hex")
    hcells = (128, 64, 64) if args.workload != "beam_s" else (32, 16, 16)
    lin = np.load(os.path.join(GOLDEN, "hex_p1_nh.npz"))
    xi1 = meshes.local_pattern(lin["points"], lin["elements"], 0, "hex")
    Ph, elh = meshes.structured_hex(hcells, (2.0, 1.0, 1.0), xi1)   # linear hexes
    Phd, elhd = torch.from_numpy(Ph).cuda(), torch.from_numpy(elh).cuda()
    for _ in range(args.warmup):
        Xh3, Eh3 = meshes.raise_hex_order_device(Phd, elhd, xi)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(steps):
        Xh3, Eh3 = meshes.raise_hex_order_device(Phd, elhd, xi)
    e1.record()
    torch.cuda.synchronize()
    ms_h = e0.elapsed_time(e1) / steps
    hexes = dict(workload="structured box %dx%dx%d linear hexes on 2x1x1 -> p=3 (64-node Gauss-Lobatto layout)"
                          % hcells, nelem=int(elh.shape[0]), nnode=int(Xh3.shape[0]), ms_per_step=ms_h,
                 melem_s=elh.shape[0] / (ms_h * 1e-3) / 1e6,
                 note="each call counts the nodes first and allocates the outputs (two calls of the C entry point)")
    del Xh3, Eh3
    line = dict(metric="high-order tet mesh generation rate (linear tets raised to p=3 per second)", value=value,
                unit="Melem/s", n_gpus=1, steps=steps, warmup=args.warmup, ms_per_step=ms, higher_is_better=True,
                scaling="weak", vs_baseline=None, dtype="int64+f64", data="synthetic",
                config=dict(workload="Kuhn-split box %dx%dx%d cubes on 2x1x1, %d tets, %d vertices -> %d nodes "
                                     "(equispaced p=3, 20 nodes per tet)" % (cells + (nelem, nvert, nnode)),
                            inputs="larger than L2 (outputs %.2f GB)" % ((8 * npe * nelem + 24 * nnode) / 1e9)),
                roofline=dict(bound="hbm", achieved=nbytes / (ms * 1e-3) / 1e9, peak=hbm, unit="GB/s",
                              frac=nbytes / (ms * 1e-3) / 1e9 / hbm, traffic=None, bytes_min_per_step=nbytes,
                              peak_source="MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback"),
                e2e=e2e, cpu_baseline=cpu, gpu_launches=launches * steps, clocks=clk.summary(), hex=hexes)
    print(json.dumps(line), flush=True)


def _time_device(fn, steps, warmup=3):
    """Mean device time (ms) of fn() over `steps` calls after `warmup`, CUDA events on the current
    stream, with nvidia-smi clock samples over the timed calls."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps, clk.summary()


def run_dpf(args):
    """Electromechanics (displacement-potential, nvar 4) assembly of IsotropicElectroMechanics_108
    (mu1 = 0.4, mu2 = 0.2, lambda = 15, eps_2 = 1.5, the golden case's parameters): the tet p=2 beam
    (48x12x12 jittered lattice, Delaunay, 8 Gauss points) and a structured p=2 hex box (40x32x32,
    27 Gauss points), CSR by row search plus the FP64 residual; deformation and potential seeded and
    smooth. One step = zero the outputs and assemble."""
    import torch
    from florence_gb300 import meshes
    from florence_gb300.electromechanics import DPFAssembler
    res = {}
    for kind in ("tet_p2", "hex_p2"):
        g = np.load(os.path.join(GOLDEN, "dpf_%s_em108.npz" % kind))
        if kind == "tet_p2":
            pat = meshes.local_pattern(g["points"], g["elements"], 0, "tet")
            cells = (48, 12, 12) if args.workload != "beam_s" else (24, 6, 6)
            P, el = meshes.jittered_tet_beam(cells, (4.0, 1.0, 1.0), 1, pat)
        else:
            pat = meshes.local_pattern(g["points"], g["elements"], 0, "hex")
            cells = (40, 32, 32) if args.workload != "beam_s" else (20, 16, 16)
            P, el = meshes.structured_hex(cells, (4.0, 1.0, 1.0), pat)
        x = P + smooth_displacement(P, seed=2)
        phi = 0.1 * np.sin(np.pi * P[:, 0] / 4.0) * np.cos(np.pi * P[:, 1])
        asm = DPFAssembler(P, el, g["Jm"], g["AllGauss"], tuple(g["params"]), material=str(g["material"]),
                           mode="squeeze")
        xd, pd = torch.from_numpy(x).cuda(), torch.from_numpy(phi).cuda()
        V = torch.zeros(asm.nnz, dtype=torch.float64, device="cuda")
        T = torch.zeros(asm.nnode * 4, dtype=torch.float64, device="cuda")

        def step():
            V.zero_()
            T.zero_()
            asm.assemble(xd, pd, V=V, T=T)
        ms, clocks = _time_device(step, max(3, min(args.steps, 20)))
        asm.check_flags("dpf bench")
        nq = int(np.ravel(g["AllGauss"]).shape[0])
        res[kind] = dict(nelem=int(el.shape[0]), nnode=int(P.shape[0]), nnz=int(asm.nnz), gauss_points=nq,
                         ms_per_step=ms, melem_s=el.shape[0] / (ms * 1e-3) / 1e6, clocks=clocks,
                         bytes_min=int(8 * 4 * P.shape[0] * 2 + 8 * asm.nnz + 8 * 4 * P.shape[0]))
        del asm, V, T
        torch.cuda.empty_cache()
    line = dict(metric="electromechanics (DPF, nvar 4) FP64 assembly throughput, tet p=2 beam", unit="Melem/s",
                value=res["tet_p2"]["melem_s"], n_gpus=1, steps=max(3, min(args.steps, 20)), warmup=3,
                higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f64", data="synthetic",
                config=dict(workload="IsotropicElectroMechanics_108 (mu1 0.4, mu2 0.2, lambda 15, eps_2 1.5): tet p=2 "
                                     "beam 48x12x12 jittered Delaunay and p=2 hex box 40x32x32, CSR by row search + "
                                     "residual"), tet_p2=res["tet_p2"], hex_p2=res["hex_p2"],
                clocks=res["tet_p2"]["clocks"])
    print(json.dumps(line), flush=True)


def run_mass(args):
    """Consistent mass sum_g rho N_a N_b w |det dX/dxi| on the nvar diagonal (fl_ConsistentMass) of the
    tet p=3 beam (47 535 elements, 14 Gauss points) into its CSR pattern, through the element-to-nonzero
    maps and by row search; and the lumped mass."""
    import torch
    import florence_gb300 as fl
    W = workload(args.workload)
    g = np.load(os.path.join(GOLDEN, "tet_p3_mr_jitter.npz"))
    res = {}
    asm = fl.DeviceAssembler(W["points"], W["elements"], W["Jm"], W["w"], "NeoHookean", (1.0, 10.0), mode="csr",
                             Bases=g["Bases"])
    sq = fl.DeviceAssembler(W["points"], W["elements"], W["Jm"], W["w"], "NeoHookean", (1.0, 10.0), mode="squeeze",
                            Bases=g["Bases"], sparsity=(asm.indices, asm.indptr, None, None))
    V = torch.zeros(asm.nnz, dtype=torch.float64, device="cuda")
    M = torch.zeros(asm.nnode * 3, dtype=torch.float64, device="cuda")
    steps = max(3, min(args.steps, 20))
    for name, a in (("maps", asm), ("row_search", sq)):
        def step(a=a):
            V.zero_()
            a.consistent_mass(1.0, V=V)
        ms, clocks = _time_device(step, steps)
        a.check_flags("mass bench")
        res[name] = dict(ms_per_step=ms, melem_s=W["elements"].shape[0] / (ms * 1e-3) / 1e6, clocks=clocks)

    def lumped():
        M.zero_()
        asm.lumped_mass(1.0, M=M)
    ms, clocks = _time_device(lumped, steps)
    res["lumped"] = dict(ms_per_step=ms, melem_s=W["elements"].shape[0] / (ms * 1e-3) / 1e6)
    nnz = asm.nnz
    peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    bmin = 8 * nnz + 4 * W["elements"].size + 8 * 3 * W["points"].shape[0]
    line = dict(metric="consistent mass assembly throughput (CSR, element-to-nonzero maps)", unit="Melem/s",
                value=res["maps"]["melem_s"], n_gpus=1, steps=steps, warmup=3, higher_is_better=True,
                scaling="weak", vs_baseline=None, dtype="f64", data="synthetic",
                config=dict(W["desc"], nelem=int(W["elements"].shape[0]), nnz=int(nnz)),
                roofline=dict(bound="hbm", achieved=bmin / (res["maps"]["ms_per_step"] * 1e-3) / 1e9, peak=hbm,
                              unit="GB/s", frac=bmin / (res["maps"]["ms_per_step"] * 1e-3) / 1e9 / hbm,
                              bytes_min_per_launch=bmin,
                              peak_source="MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback"),
                maps=res["maps"], row_search=res["row_search"], lumped=res["lumped"], clocks=res["maps"]["clocks"])
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="beam", choices=["beam", "beam_s", "cube"])
    ap.add_argument("--arith", default="reference_tensor",
                    choices=["fp64", "float_pair", "tensor", "reference_tensor", "mixed"],
                    help="arithmetic of the stiffness contraction (the default: FP64 tangent as tensor-core GEMMs "
                         "against the reference tensor; FP64, float pairs on the FP32 pipe, the per-element digit "
                         "split, or the split-BF16 tensor-core tangent with FP32 values)")
    ap.add_argument("--tc-tiling", default="0,0",
                    help="tile group and reduction chunk of the split-BF16 kernel (0,0 = automatic)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle check of the timed workload")
    ap.add_argument("--newton", action="store_true", help="Newton load stepping of the beam instead")
    ap.add_argument("--explicit", action="store_true", help="explicit dynamics of the hex beam instead")
    ap.add_argument("--explicit-steps", type=int, default=10000)
    ap.add_argument("--tangent", default="fp64", choices=["fp64", "mixed", "hybrid", "both", "all"],
                    help="Newton Jacobian (both: FP64 then mixed; all: FP64, mixed, hybrid; with the "
                         "differences of the solutions)")
    ap.add_argument("--newton-max-iter", type=int, default=25,
                    help="Newton iterations per increment before failing (small values give a short profile run)")
    ap.add_argument("--forcing", default="ew", choices=["ew", "rel"],
                    help="PCG tolerance per Newton step: Eisenstat-Walker, or 0.1 x relative residual")
    ap.add_argument("--spmv", default="split", choices=["split", "fp64"],
                    help="PCG product for FP64 tangents: float-pair split on the FP32 pipe, or FP64")
    ap.add_argument("--linear", default="pmg", choices=["pcg", "pmg"],
                    help="Newton's linear step: flexible CG with the two-level p-multigrid cycle (the default; FP64 "
                         "tangent), or block-Jacobi PCG (any tangent)")
    ap.add_argument("--pcg-loop", default="device", choices=["device", "host"],
                    help="PCG iterations as one CUDA graph with a device-side loop, or launched from the host")
    ap.add_argument("--pcg", action="store_true", help="PCG iterations on the beam's tangent instead")
    ap.add_argument("--pcg-iters", type=int, default=400)
    ap.add_argument("--batched", action="store_true", help="batched uneven instances instead")
    ap.add_argument("--instances", type=int, default=512)
    ap.add_argument("--batch-gb", type=float, default=40.0, help="CSR memory budget per sub-batch")
    ap.add_argument("--warmstart", action="store_true", help="learned warm start on the plate instead")
    ap.add_argument("--meshing", action="store_true", help="device high-order tet mesh generation instead")
    ap.add_argument("--dpf", action="store_true", help="electromechanics (nvar 4) assembly instead")
    ap.add_argument("--mass", action="store_true", help="consistent and lumped mass assembly instead")
    ap.add_argument("--ws-train", type=int, default=2000, help="training solves")
    ap.add_argument("--ws-test", type=int, default=200, help="held-out solves")
    ap.add_argument("--ws-increments", type=int, default=5)
    ap.add_argument("--ws-steps", type=int, default=20000, help="Adam steps of the network")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.pcg_loop == "host" and args.impl != "reference":
        from florence_gb300.newton import set_pcg_device_loop
        set_pcg_device_loop(False)
    if args.impl == "reference":
        run_reference(args)
    elif args.newton:
        run_newton(args)
    elif args.pcg:
        run_pcg(args)
    elif args.explicit:
        run_explicit(args)
    elif args.batched:
        run_batched(args)
    elif args.warmstart:
        run_warmstart(args)
    elif args.meshing:
        run_meshing(args)
    elif args.dpf:
        run_dpf(args)
    elif args.mass:
        run_mass(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
