"""Benchmark of the GB300 direct J/K Fock build.

Workload (one "step" = one full RHF J+K Fock build): a seeded (H2O)32 cluster
in a 14 A cube, cc-pVDZ with spherical d (768 basis functions), density
D = 2 C C^T from 160 Loewdin-orthonormalised random columns, Schwarz / density
screening threshold 1e-10.

  value  builds/s with D and F resident in device memory (C-ABI device entry)
  e2e    builds/s through OpenQP's seam routec_fock_jk with host buffers
         (H2D of D and D2H of F inside every timed step)
  roofline  FP64 roofline of the dominant class kernel: algorithmic flops
            (3 R N_c per primitive quartet + digestion) / its event-timed
            duration, against the measured FP64 FMA peak of this device
  cpu_baseline  the oracle (CPU restatement of OpenQP's int2 path, OpenMP, all
            host cores) on a bounded sample: the shell pairs of one rank of a
            round-robin split of the cost-sorted pair list, plus the Schwarz
            set-up the reference repeats in every fock_jk call.

--impl reference times that CPU implementation alone (rank 0 only).
Multi-GPU runs are independent replicas (one molecule per rank, no collective).
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # the headline workload (the metric's configuration)
    # traffic: DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per build of the
    # dominant class, scaled by quartets from a one-launch ncu capture of the same kernel on
    # (H2O)16 6-31G(d): 15.02 MB for 1 648 969 (ss|sp) quartets, 9.11 bytes each (the 8-byte list
    # entry; pairs and densities stay in L2), x 34 830 594 quartets here
    "water32_ccpvdz": dict(name="(H2O)32 cc-pVDZ spherical RHF J+K Fock build", nwater=32, edge=14.0, seed=0,
                           basis="cc-pvdz", cutoff=1e-10, traffic={"(ss|sp)": 317.2e6}),
    # the plain-FP64 parity configuration
    "water4_631gd": dict(name="(H2O)4 6-31G(d) Cartesian RHF J+K Fock build", nwater=4, edge=6.0, seed=0,
                         basis="6-31g(d)", cutoff=1e-10),
    # small cases for profiling
    "water8_ccpvdz": dict(name="(H2O)8 cc-pVDZ spherical RHF J+K Fock build", nwater=8, edge=8.82, seed=0,
                          basis="cc-pvdz", cutoff=1e-10),
    "water16_631gd": dict(name="(H2O)16 6-31G(d) Cartesian RHF J+K Fock build", nwater=16, edge=9.52, seed=0,
                          basis="6-31g(d)", cutoff=1e-10),
    # linear all-trans C40H82, 6-31G(d) Cartesian (the precision-split configuration)
    "alkane40_631gd": dict(name="C40H82 6-31G(d) Cartesian RHF J+K Fock build", alkane=40, seed=0,
                           basis="6-31g(d)", cutoff=1e-10),
    # 256 water clusters of 1-16 molecules (uniform), 6-31G, built together
    "batch256_631g": dict(name="256 water clusters (1-16 H2O, uniform), 6-31G, batched RHF J+K builds", batch=256,
                          seed=0, basis="6-31g", cutoff=1e-10),
    # full direct SCF (RHF, DIIS, |dE| < 1e-9) of the headline cluster: builds/s inside the SCF
    "scf_water32_ccpvdz": dict(name="(H2O)32 cc-pVDZ spherical RHF direct SCF (dE 1e-9, DIIS)", nwater=32, edge=14.0,
                               seed=0, basis="cc-pvdz", cutoff=1e-10, scf=True),
    # the precision-split configuration over a whole SCF: FP64 full builds vs mixed + incremental
    "scf_alkane40_631gd": dict(name="C40H82 6-31G(d) RHF SCF: mixed precision + incremental dD vs plain FP64",
                               alkane=40, seed=0, basis="6-31g(d)", cutoff=1e-10, scf=True, mixed_scf=True),
    # the differentiation configuration: two-electron gradient of (H2O)16 6-31G(d)
    "grad_water16_631gd": dict(name="(H2O)16 6-31G(d) Cartesian RHF two-electron gradient (grd2)", nwater=16,
                               edge=9.52, seed=0, basis="6-31g(d)", cutoff=1e-10, grad=True),
    # the MRSF two-electron gradient (routec_grad2_mrsf): grd2 with the eleven-matrix MRSF density
    "grad_mrsf_water16_631gd": dict(name="(H2O)16 6-31G(d) Cartesian MRSF two-electron gradient (grd2 with the "
                                         "grd2_mrsf_compute_data_t density)", nwater=16, edge=9.52, seed=0,
                                    basis="6-31g(d)", cutoff=1e-10, grad=True, mrsf_grad=True),
    # f shells: (H2O)16 cc-pVTZ spherical (one f shell per O, d on H; 928 bf)
    "water16_ccpvtz": dict(name="(H2O)16 cc-pVTZ spherical RHF J+K Fock build (f shells)", nwater=16, edge=9.52,
                           seed=0, basis="cc-pvtz", cutoff=1e-10),
    # response-type (TDHF A+B and A-B) builds: 8 trial transition densities per build
    "td_water16_631gd": dict(name="(H2O)16 6-31G(d) Cartesian TDHF A+B and A-B build, 8 trial vectors", nwater=16,
                             edge=9.52, seed=0, basis="6-31g(d)", cutoff=1e-10, td=True, nvec=8),
    "td_water32_ccpvdz": dict(name="(H2O)32 cc-pVDZ spherical TDHF A+B and A-B build, 8 trial vectors", nwater=32,
                              edge=14.0, seed=0, basis="cc-pvdz", cutoff=1e-10, td=True, nvec=8),
    # the MRSF Davidson sigma session (routec_sig_iter): 8 new trial vectors of a triplet-reference
    # (nocca = noccb + 2) singlet MRSF, MO transforms + one nmat-7 integral pass
    "mrsf_water16_631gd": dict(name="(H2O)16 6-31G(d) Cartesian MRSF singlet sigma session, 8 trial vectors "
                                    "(nocca 81, noccb 79)", nwater=16, edge=9.52, seed=0, basis="6-31g(d)",
                               cutoff=1e-10, sigma=True, nvec=8, mrst=1),
    # CAM (range-separated) RHF build of the headline cluster: CAM-B3LYP's alpha, beta, mu
    "cam_water32_ccpvdz": dict(name="(H2O)32 cc-pVDZ spherical RHF CAM J+K build (alpha 0.19, beta 0.46, mu 0.33)",
                               nwater=32, edge=14.0, seed=0, basis="cc-pvdz", cutoff=1e-10,
                               cam=(0.19, 0.46, 0.33, 1.0, 0.0)),
    # (dd|dd) only: one Cartesian d shell (6-31G(d) carbon d, exponent 0.8) on each
    # point of a 4 x 4 x 4 cubic lattice of spacing 1.54 A, so that all 2080 pairs overlap
    "dd_only": dict(name="(dd|dd)-only: 64 Cartesian d shells (exponent 0.8) on a 4x4x4 lattice, 1.54 A spacing",
                    lattice=4, spacing=1.54, dexp=0.8, seed=0, cutoff=1e-10),
}
WORKLOAD = dict(WORKLOADS["water32_ccpvdz"])

# What the CPU baseline runs: the oracle restates OpenQP's int2 quartet loop
# (screening, digestion, OpenMP over cost-sorted shell pairs) but evaluates
# every class by Rys quadrature, where OpenQP evaluates quartets with max L <= 2
# by its rotated-axis engine with Boys-function tables (int2.F90:1079-1107).
ENGINE_FOCK = ("oracle port of OpenQP's int2 loop with Rys quadrature for every class; OpenQP's own binary uses its "
               "rotated-axis engine for max L <= 2 (int2.F90:1079-1107), so this is not the reference binary's speed")
ENGINE_GRAD = "oracle port of OpenQP's grd2 with Rys derivative integrals, as grd2_rys.F90 (not the reference binary)"


def make_workload(overlap="library"):
    """Basis and seeded density of the workload.  The overlap for the Loewdin
    step comes from the library's host routine, or from the oracle in the
    reference arm (identical to 1e-14)."""
    from openqp_gb300 import workloads
    from openqp_gb300.basis import build_basis
    if "lattice" in WORKLOAD:
        bas = workloads.d_lattice(WORKLOAD["lattice"], WORKLOAD["spacing"], WORKLOAD["dexp"])
    elif "alkane" in WORKLOAD:
        z, xyz = workloads.alkane(WORKLOAD["alkane"], WORKLOAD["seed"])
        bas = build_basis(z, xyz, WORKLOAD["basis"])
    else:
        bas = workloads.water_cluster_basis(WORKLOAD["nwater"], WORKLOAD["edge"], WORKLOAD["seed"],
                                            WORKLOAD["basis"])
    if "lattice" in WORKLOAD:
        nocc = bas.nbf // 4
    else:
        nocc = workloads.nelectrons(bas) // 2
    if overlap == "library":
        from openqp_gb300.onee import one_electron
        S = one_electron(bas)[0]
    else:
        from oracle import oracle
        oracle.build()
        S = oracle.Oracle(bas, cutoff=WORKLOAD["cutoff"]).one_electron("S")
    d = workloads.density(bas, nocc, WORKLOAD["seed"], S=S)
    return bas, d


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x):
    """The largest value of x over the ranks of the process group (one rank:
    x).  NCCL groups reduce on the GPU, gloo groups on the host."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(prefix="oqpg_clocks_%d_" % self.gpu, suffix=".csv")
            self.fh = os.fdopen(fd, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        lines = open(self.path).read().splitlines()
        try:
            os.remove(self.path)
        except OSError:
            pass
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in lines:
            p = [v.strip() for v in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = max(mx, float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def sampled(run, budget_s):
    """Bounded sample of a quartet loop over the cost-sorted bra pairs.
    run(stride, offset) times the loop over the pairs p with p % stride ==
    offset and returns (loop seconds, info).  The stride is refined until the
    sample fills at least half the budget (or is the whole loop); the timed
    sample takes the middle pair of every stride (offset stride // 2), since
    the first pair of the cost-sorted order is the heaviest and offset 0
    over-weights it.  Returns (estimated full loop seconds, stride, info)."""
    stride = 997
    for _ in range(6):
        t, info = run(stride, stride // 2)
        if stride == 1 or t >= 0.5 * budget_s:
            break
        stride = max(1, int(stride * max(t, 1e-3) / budget_s))
    return t * stride, stride, info


def cpu_baseline(bas, d, budget_s=20.0):
    """Oracle on a bounded sample; returns builds/s and a description."""
    from oracle import oracle
    oracle.build()
    o = oracle.Oracle(bas, cutoff=WORKLOAD["cutoff"])
    cores = os.cpu_count()
    t0 = time.perf_counter()
    q = o.schwarz(nthreads=cores)
    t_schwarz = time.perf_counter() - t0

    def run(stride, offset):
        _, st = o.fock_jk_sample(d, stride, offset, nthreads=cores, schwarz=q)
        return st["t_twoei"], st

    t_loop, stride, st = sampled(run, budget_s)
    t_build = t_loop + st["t_init"] + t_schwarz
    return dict(value=1.0 / t_build, unit="builds/s", cores=cores, kind="port", engine=ENGINE_FOCK,
                sample="oracle fock_jk over 1/%d of the cost-sorted shell pairs (the middle pair of every %d), x%d, "
                       "plus the full Schwarz set-up (%.2f s) the reference repeats per build; %d quartets in the sample"
                       % (stride, stride, stride, t_schwarz, st["quartets"])), dict(sample_s=t_loop / stride,
                                                                                   stride=stride)


def td_workload(overlap="library"):
    """Basis and the seeded (nvec, nbf, nbf) transition densities of a TD workload."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(WORKLOAD["nwater"], WORKLOAD["edge"], WORKLOAD["seed"], WORKLOAD["basis"])
    if overlap == "library":
        from openqp_gb300.onee import one_electron
        S = one_electron(bas)[0]
    else:
        from oracle import oracle
        oracle.build()
        S = oracle.Oracle(bas, cutoff=WORKLOAD["cutoff"]).one_electron("S")
    x = workloads.transition_densities(bas, workloads.nelectrons(bas) // 2, WORKLOAD["nvec"], WORKLOAD["seed"], S=S)
    return bas, x


def cpu_baseline_td(bas, x, budget_s):
    """The oracle's int2_td_data_t restatement (all host cores) over 1/stride
    of the bra shell pairs, scaled by stride, plus its full set-up."""
    from oracle import oracle
    oracle.build()
    o = oracle.Oracle(bas, cutoff=WORKLOAD["cutoff"])
    cores = os.cpu_count()

    def run(stride, offset):
        _, _, st = o.fock_td_sample(x, 3, stride, offset, nthreads=cores)
        return st["t_twoei"], st

    t_loop, stride, st = sampled(run, budget_s)
    t = t_loop + st["t_setup"]
    return {"value": 1.0 / t, "unit": "TD builds/s", "cores": cores, "kind": "port", "engine": ENGINE_FOCK,
            "sample": "oracle int2_td_data_t restatement (A+B and A-B, %d vectors) over 1/%d of the cost-sorted bra "
                      "shell pairs (the middle pair of every stride), x%d, plus the work outside the quartet loop "
                      "(set-up, reduction; %.2f s); %d quartets in the sample"
                      % (x.shape[0], stride, stride, st["t_setup"], st["quartets"])}


def run_td(args):
    """TD builds/s: A+B and A-B of nvec trial transition densities in one
    pass over the quartets (OpenQP's int2_td_data_t with int_apb and int_amb),
    densities resident on the device; e2e through the host-buffer entry."""
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    from openqp_gb300 import build as bld
    bld.build()
    from openqp_gb300.fock import NCLASS, FockBuilder, class_flops, class_labels, fp64_peak_tflops
    bas, x = td_workload()
    nvec = x.shape[0]
    fb = FockBuilder(bas, cutoff=WORKLOAD["cutoff"])
    fb.set_precision(args.precision, args.mixed_threshold)
    xt = torch.from_numpy(x).cuda()
    st = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        fb.fock_td_device(xt, apb=True, amb=True, stream=st)
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    times, stats = [], []
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        pa, ma = fb.fock_td_device(xt, apb=True, amb=True, stream=st)
        e1.record(st)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
        stats.append(fb.stats())
    clocks = sampler.stop()
    tsum = max_over_ranks(sum(times) / 1000.0)
    value = ws * args.steps / tsum
    e2e_t = []
    if not args.no_e2e:
        fb.fock_td(x, apb=True, amb=True)
        for _ in range(args.steps):
            t0 = time.perf_counter()
            hp, hm = fb.fock_td(x, apb=True, amb=True)
            e2e_t.append(time.perf_counter() - t0)
        assert np.abs(hp - pa.cpu().numpy()).max() < 1e-12
    e2e = ws * args.steps / max_over_ranks(sum(e2e_t)) if e2e_t else float("nan")
    labels = class_labels()
    ms = np.mean([s["ms_per_class"] for s in stats], axis=0)
    cdom = int(np.argmax(ms))
    s0 = stats[-1]
    pure = bool(bas.harmonic.any())
    fl = [class_flops(c, s0["prim_per_class"][c], s0["per_class"][c], nk=2 * nvec, nj=nvec, pure=pure)
          for c in range(NCLASS)]
    achieved = fl[cdom] / (ms[cdom] * 1e-3) / 1e12
    peak = fp64_peak_tflops()
    nb = int(8 * nvec * bas.nbf * bas.nbf)
    line = {"metric": "TDHF A+B / A-B builds/s (%d trial vectors per build)" % nvec, "value": value,
            "unit": "TD builds/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * tsum / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else args.precision,
            "data": "synthetic (seeded water cluster, seeded unit-norm transition densities C_occ Y C_vir^T)",
            "config": {"workload": WORKLOAD["name"], "nbf": bas.nbf, "nvec": nvec, "cutoff": WORKLOAD["cutoff"],
                       "flags": "int_apb + int_amb", "l2": "flushed (256 MB write) before every timed step"},
            "e2e": {"value": e2e, "unit": "TD builds/s", "h2d_bytes_per_step": nb, "d2h_bytes_per_step": 2 * nb},
            "roofline": {"bound": "fp64", "kernel": labels[cdom], "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                         "peak_source": "measured: FP64 FMA-chain probe on this device",
                         "kernel_ms": float(ms[cdom]), "build_fp64_tflops": sum(fl) / (tsum / args.steps) / 1e12},
            "quartets_per_s": s0["quartets"] / (tsum / args.steps),
            "prim_quartets_per_s": s0["prim_quartets"] / (tsum / args.steps),
            "gpu_launches": int(sum(s["launches"] for s in stats)), "clocks": clocks,
            "class_ms": {labels[c]: round(float(ms[c]), 3) for c in range(NCLASS) if ms[c] > 0},
            "list_ms": s0["list_ms"]}
    if not args.no_cpu and rank == 0:
        line["cpu_baseline"] = cpu_baseline_td(bas, x, args.cpu_budget)
    if rank == 0:
        print(json.dumps(line), flush=True)


def sigma_workload(overlap="library"):
    """Basis, occupations and the seeded session inputs of the sigma workload."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(WORKLOAD["nwater"], WORKLOAD["edge"], WORKLOAD["seed"], WORKLOAD["basis"])
    if overlap == "library":
        from openqp_gb300.onee import one_electron
        S = one_electron(bas)[0]
    else:
        from oracle import oracle
        oracle.build()
        S = oracle.Oracle(bas, cutoff=WORKLOAD["cutoff"]).one_electron("S")
    nel = workloads.nelectrons(bas)
    na, nb = nel // 2 + 1, nel // 2 - 1
    C, fa, fb, b = workloads.mrsf_session_inputs(bas, na, nb, WORKLOAD["nvec"], WORKLOAD["seed"], S=S)
    return bas, na, nb, C, fa, fb, b


def cpu_baseline_sigma(bas, na, nb, C, fa, fb, b, budget_s):
    """The oracle's restatement of the native sigma triple: the NumPy MO
    transforms (mrsfcbc, mrsfmntoia, mrsfesum) timed whole, the nmat-7
    int2_mrsf_data_t build (all host cores) over 1/stride of the cost-sorted
    bra pairs, scaled, plus its set-up."""
    from oracle import oracle
    from oracle import mrsf_sigma as ms
    oracle.build()
    o = oracle.Oracle(bas, cutoff=WORKLOAD["cutoff"])
    cores = os.cpu_count()
    mrst = WORKLOAD["mrst"]
    n = bas.nbf
    t0 = time.perf_counter()
    xs = [ms.iatogen(b[:, v], n, na, nb) for v in range(b.shape[1])]
    d3 = np.stack([ms.mrsfcbc(C, C, x, na, nb, mrst) for x in xs])
    t_cbc = time.perf_counter() - t0

    def run(stride, offset):
        f3, st = o.fock_mrsf_sample(d3, stride, offset, nthreads=cores)
        return st["t_twoei"], (st, f3)

    t_loop, stride, (st, f3) = sampled(run, budget_s)
    t0 = time.perf_counter()
    for v in range(b.shape[1]):
        ms.mrsfmntoia(f3[v], C, C, na, nb, mrst) + ms.mrsfesum(xs[v], fa, fb, na, nb, mrst)
    t_back = time.perf_counter() - t0
    t = t_loop + st["t_setup"] + t_cbc + t_back
    return {"value": 1.0 / t, "unit": "sigma calls/s", "cores": cores, "kind": "port", "engine": ENGINE_FOCK,
            "sample": "oracle restatement of the native MRSF sigma triple for %d vectors: NumPy mrsfcbc / "
                      "mrsfmntoia / mrsfesum timed whole (%.2f s), the int2_mrsf_data_t quartet loop over 1/%d of the "
                      "cost-sorted bra shell pairs (the middle pair of every stride), x%d, plus its set-up (%.2f s); "
                      "%d quartets in the sample"
                      % (b.shape[1], t_cbc + t_back, stride, stride, st["t_setup"], st["quartets"])}


def run_sigma(args):
    """MRSF sigma calls/s: one routec_sig_iter product (A-B) X of nvec new trial
    vectors (MO -> AO, one nmat-7 integral pass, AO -> MO), device buffers
    for value, the host-buffer seam itself for e2e."""
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    from openqp_gb300 import build as bld
    bld.build()
    from openqp_gb300._lib import lib
    from openqp_gb300.fock import (NCLASS, FockBuilder, class_flops, class_labels, fp64_peak_tflops, routec_finalize,
                                   routec_init, routec_sig_init, routec_sig_iter, routec_sig_set_scale)
    bas, na, nb, C, fa, fb, b = sigma_workload()
    nvec, mrst = b.shape[1], WORKLOAD["mrst"]
    if routec_init(bas, WORKLOAD["cutoff"]) != 0:
        raise RuntimeError("routec_fock_init failed")
    rc = routec_sig_init(C, C, fa, fb, na, nb, mrst)
    if rc:
        raise RuntimeError("routec_sig_init returned %d" % rc)
    routec_sig_set_scale(1.0)
    bt = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()      # column v contiguous = Fortran (ntrial, nv)
    out = torch.empty_like(bt)
    st = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def call():
        rc = lib().oqpg_sig_iter_device(ctypes.c_void_p(bt.data_ptr()), nvec, ctypes.c_void_p(out.data_ptr()),
                                        ctypes.c_void_p(st.cuda_stream))
        if rc:
            raise RuntimeError("oqpg_sig_iter_device returned %d" % rc)

    for _ in range(args.warmup):
        call()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    times = []
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        call()
        e1.record(st)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    clocks = sampler.stop()
    tsum = max_over_ranks(sum(times) / 1000.0)
    value = ws * args.steps / tsum
    e2e_t = []
    if not args.no_e2e:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            sg, info = routec_sig_iter(b)
            e2e_t.append(time.perf_counter() - t0)
            if info:
                raise RuntimeError("routec_sig_iter returned %d" % info)
        assert np.abs(sg - out.cpu().numpy().T).max() < 1e-12 * max(1.0, np.abs(sg).max())
    e2e = ws * args.steps / max_over_ranks(sum(e2e_t)) if e2e_t else float("nan")
    # the integral pass alone (same seven densities per vector) for the class times and the roofline
    fbld = FockBuilder(bas, cutoff=WORKLOAD["cutoff"])
    from oracle import mrsf_sigma as ms
    d3 = np.stack([ms.mrsfcbc(C, C, ms.iatogen(b[:, v], bas.nbf, na, nb), na, nb, mrst) for v in range(nvec)])
    fbld.fock_mrsf(d3)
    fbld.fock_mrsf(d3)
    s0 = fbld.stats()
    labels = class_labels()
    ms_c = np.array(s0["ms_per_class"])
    cdom = int(np.argmax(ms_c))
    pure = bool(bas.harmonic.any())
    nk, nj = 2 * 7 * nvec, 4 * nvec
    fl = [class_flops(c, s0["prim_per_class"][c], s0["per_class"][c], nk=nk, nj=nj, pure=pure) for c in range(NCLASS)]
    achieved = fl[cdom] / (ms_c[cdom] * 1e-3) / 1e12
    peak = fp64_peak_tflops()
    routec_finalize()
    nbytes = int(8 * b.size)
    line = {"metric": "MRSF sigma calls/s (%d trial vectors per call)" % nvec, "value": value,
            "unit": "sigma calls/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * tsum / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded water cluster, Loewdin MO set, orbital-energy ladder MO Fock, seeded unit "
                    "trial vectors)",
            "config": {"workload": WORKLOAD["name"], "nbf": bas.nbf, "nvec": nvec, "nocca": na, "noccb": nb,
                       "kind": "singlet" if mrst == 1 else "triplet", "cutoff": WORKLOAD["cutoff"],
                       "l2": "flushed (256 MB write) before every timed step"},
            "e2e": {"value": e2e, "unit": "sigma calls/s", "h2d_bytes_per_step": nbytes,
                    "d2h_bytes_per_step": nbytes},
            "roofline": {"bound": "fp64", "kernel": labels[cdom] + " (the call's integral pass)",
                         "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                         "traffic": None, "peak_source": "measured: FP64 FMA-chain probe on this device",
                         "kernel_ms": float(ms_c[cdom]), "integral_pass_ms": float(s0["total_ms"])
                         if "total_ms" in s0 else None},
            # per call: the integral pass's launches (as counted by the same job on a FockBuilder) plus the
            # session's four elementwise kernels; the cuBLAS DGEMMs are library kernels and not counted
            "gpu_launches": int(args.steps * (s0["launches"] + 4)), "clocks": clocks,
            "class_ms": {labels[c]: round(float(ms_c[c]), 3) for c in range(NCLASS) if ms_c[c] > 0}}
    if not args.no_cpu and rank == 0:
        line["cpu_baseline"] = cpu_baseline_sigma(bas, na, nb, C, fa, fb, b, args.cpu_budget)
    if rank == 0:
        print(json.dumps(line), flush=True)


def cpu_baseline_cam(bas, d, budget_s):
    """The oracle's two-pass CAM build (all host cores) over 1/stride of the
    cost-sorted bra pairs, scaled, plus the work outside the quartet loops."""
    from oracle import oracle
    oracle.build()
    o = oracle.Oracle(bas, cutoff=WORKLOAD["cutoff"])
    cores = os.cpu_count()
    cam = WORKLOAD["cam"]

    def run(stride, offset):
        _, st = o.fock_jk_cam_sample(d, *cam[:3], stride, offset, *cam[3:], nthreads=cores)
        return st["t_twoei"], st

    t_loop, stride, st = sampled(run, budget_s)
    t = t_loop + (st["t_total"] - st["t_twoei"])
    return {"value": 1.0 / t, "unit": "builds/s", "cores": cores, "kind": "port", "engine": ENGINE_FOCK,
            "sample": "oracle two-pass CAM build (1/r and erf(mu r)/r, own Schwarz bounds) over 1/%d of the "
                      "cost-sorted bra shell pairs (the middle pair of every stride), x%d, plus set-up; %d quartets "
                      "in the sample"
                      % (stride, stride, st["quartets"])}


def run_cam(args):
    """CAM builds/s: OpenQP's int2_run_cam (1/r pass, erf(mu r)/r pass with its
    own Schwarz bounds) of the workload density, device-resident; e2e through
    routec_fock_jk_cam with host buffers."""
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    from openqp_gb300 import build as bld
    bld.build()
    from openqp_gb300._lib import lib
    from openqp_gb300.fock import FockBuilder, cam_array, class_flops, class_labels, fp64_peak_tflops, \
        routec_fock_jk_cam, routec_init, ptr
    bas, d = make_workload()
    fb = FockBuilder(bas, cutoff=WORKLOAD["cutoff"])
    fb.set_precision(args.precision, args.mixed_threshold)
    cam = WORKLOAD["cam"]
    ca = cam_array(*cam)
    dt = torch.from_numpy(d[None]).cuda()
    out = torch.empty_like(dt)
    st = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def build():
        rc = lib().oqpg_fock_jk_cam_device(fb.h, ctypes.c_void_p(dt.data_ptr()), ctypes.c_void_p(out.data_ptr()), 1,
                                           ptr(ca), ctypes.c_void_p(st.cuda_stream))
        if rc:
            raise RuntimeError("oqpg_fock_jk_cam_device returned %d" % rc)

    for _ in range(args.warmup):
        build()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    times = []
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        build()
        e1.record(st)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    clocks = sampler.stop()
    tsum = max_over_ranks(sum(times) / 1000.0)
    value = ws * args.steps / tsum
    # the plain (1/r only) build of the same density for comparison
    tp = []
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        fb.fock_jk_device(dt, out=out, stream=st)
        e1.record(st)
        e1.synchronize()
        tp.append(e0.elapsed_time(e1))
    stats = fb.stats()   # the last pass recorded: the plain build
    e2e_t = []
    if not args.no_e2e:
        routec_init(bas, WORKLOAD["cutoff"])
        routec_fock_jk_cam(d, bas.nbf, 1, *cam)
        for _ in range(args.steps):
            t0 = time.perf_counter()
            _, info = routec_fock_jk_cam(d, bas.nbf, 1, *cam)
            e2e_t.append(time.perf_counter() - t0)
            if info:
                raise RuntimeError("routec_fock_jk_cam returned %d" % info)
    e2e = ws * args.steps / max_over_ranks(sum(e2e_t)) if e2e_t else float("nan")
    labels = class_labels()
    ms = np.array(stats["ms_per_class"])
    cdom = int(np.argmax(ms))
    pure = bool(bas.harmonic.any())
    achieved = class_flops(cdom, stats["prim_per_class"][cdom], stats["per_class"][cdom], pure=pure) / \
        (ms[cdom] * 1e-3) / 1e12
    peak = fp64_peak_tflops()
    line = {"metric": "CAM J+K Fock builds/s", "value": value, "unit": "builds/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * tsum / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else args.precision,
            "data": "synthetic (seeded water cluster and Loewdin density)",
            "config": {"workload": WORKLOAD["name"], "nbf": bas.nbf, "cutoff": WORKLOAD["cutoff"],
                       "cam": {"alpha": cam[0], "beta": cam[1], "mu": cam[2], "alpha_coulomb": cam[3],
                               "beta_coulomb": cam[4]},
                       "l2": "flushed (256 MB write) before every timed step"},
            "e2e": {"value": e2e, "unit": "builds/s", "h2d_bytes_per_step": int(d.nbytes),
                    "d2h_bytes_per_step": int(d.nbytes)},
            "roofline": {"bound": "fp64", "kernel": labels[cdom] + " (1/r pass)", "achieved": achieved,
                         "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                         "peak_source": "measured: FP64 FMA-chain probe on this device",
                         "kernel_ms": float(ms[cdom])},
            "plain_builds_per_s": args.steps / (sum(tp) / 1000.0), "clocks": clocks}
    if not args.no_cpu and rank == 0:
        line["cpu_baseline"] = cpu_baseline_cam(bas, d, args.cpu_budget)
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    if WORKLOAD.get("grad"):
        bas, d = make_workload(overlap="oracle")
        if WORKLOAD.get("mrsf_grad"):
            from openqp_gb300 import workloads
            from oracle import oracle
            oracle.build()
            S = oracle.Oracle(bas, cutoff=WORKLOAD["cutoff"]).one_electron("S")
            dm, pm, spc = workloads.mrsf_gradient_inputs(bas, WORKLOAD["seed"], S=S)
            one = lambda: cpu_baseline_grad_mrsf(bas, dm, pm, spc, args.cpu_budget)
            metric = "MRSF two-electron gradient evaluations/s"
        else:
            one = lambda: cpu_baseline_grad(bas, d, args.cpu_budget)
            metric = "two-electron gradient evaluations/s"
        vals = [one()["value"] for _ in range(max(1, args.steps))]
        cb = one()
        v = statistics.median(vals)
        cb["value"] = v
        line = {"impl": "reference", "metric": metric, "value": v, "unit": "grad evals/s", "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / v, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
                "config": {"workload": WORKLOAD["name"], "nbf": bas.nbf, "natom": bas.natom,
                           "cutoff": WORKLOAD["cutoff"]},
                "cpu_baseline": cb, "e2e": {"value": v, "unit": "grad evals/s", "h2d_bytes_per_step": 0,
                                            "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    if WORKLOAD.get("cam"):
        bas, d = make_workload(overlap="oracle")
        vals = [cpu_baseline_cam(bas, d, args.cpu_budget)["value"] for _ in range(max(1, args.steps))]
        cb = cpu_baseline_cam(bas, d, args.cpu_budget)
        v = statistics.median(vals)
        cb["value"] = v
        line = {"impl": "reference", "metric": "CAM J+K Fock builds/s", "value": v, "unit": "builds/s",
                "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / v,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded)",
                "config": {"workload": WORKLOAD["name"], "nbf": bas.nbf, "cutoff": WORKLOAD["cutoff"]},
                "cpu_baseline": cb, "e2e": {"value": v, "unit": "builds/s", "h2d_bytes_per_step": 0,
                                            "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    if WORKLOAD.get("sigma"):
        bas, na, nb, C, fa, fb, b = sigma_workload(overlap="oracle")
        vals = [cpu_baseline_sigma(bas, na, nb, C, fa, fb, b, args.cpu_budget)["value"]
                for _ in range(max(1, args.steps))]
        cb = cpu_baseline_sigma(bas, na, nb, C, fa, fb, b, args.cpu_budget)
        v = statistics.median(vals)
        cb["value"] = v
        line = {"impl": "reference", "metric": "MRSF sigma calls/s (%d trial vectors per call)" % b.shape[1],
                "value": v, "unit": "sigma calls/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1000.0 / v, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic (seeded)",
                "config": {"workload": WORKLOAD["name"], "nbf": bas.nbf, "nvec": b.shape[1], "nocca": na,
                           "noccb": nb, "cutoff": WORKLOAD["cutoff"]},
                "cpu_baseline": cb, "e2e": {"value": v, "unit": "sigma calls/s", "h2d_bytes_per_step": 0,
                                            "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    if WORKLOAD.get("td"):
        bas, x = td_workload(overlap="oracle")
        vals = [cpu_baseline_td(bas, x, args.cpu_budget)["value"] for _ in range(max(1, args.steps))]
        cb = cpu_baseline_td(bas, x, args.cpu_budget)
        v = statistics.median(vals)
        cb["value"] = v
        line = {"impl": "reference", "metric": "TDHF A+B / A-B builds/s (%d trial vectors per build)" % x.shape[0],
                "value": v, "unit": "TD builds/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1000.0 / v, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic (seeded)",
                "config": {"workload": WORKLOAD["name"], "nbf": bas.nbf, "nvec": x.shape[0],
                           "cutoff": WORKLOAD["cutoff"]},
                "cpu_baseline": cb, "e2e": {"value": v, "unit": "TD builds/s", "h2d_bytes_per_step": 0,
                                            "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    if "batch" in WORKLOAD:
        from openqp_gb300 import workloads
        from oracle import oracle
        oracle.build()
        _, bases, dens = workloads.water_batch(WORKLOAD["batch"], WORKLOAD["seed"], basis=WORKLOAD["basis"],
                                               overlap=lambda b: oracle.Oracle(b).one_electron("S"))
        vals = []
        for _ in range(max(1, args.steps)):
            cb = cpu_baseline_batch(bases, dens, args.cpu_budget)
            vals.append(cb["value"])
        v = statistics.median(vals)
        cb["value"] = v
        line = {"impl": "reference", "metric": "J+K Fock builds/s (molecule builds, batched)", "value": v,
                "unit": "builds/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1000.0 / v, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic (seeded)",
                "config": {"workload": WORKLOAD["name"], "nmol": len(bases), "cutoff": WORKLOAD["cutoff"]},
                "cpu_baseline": cb, "e2e": {"value": v, "unit": "builds/s", "h2d_bytes_per_step": 0,
                                            "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    bas, d = make_workload(overlap="oracle")
    vals = []
    info = None
    for _ in range(max(1, args.steps)):
        cb, info = cpu_baseline(bas, d, budget_s=args.cpu_budget)
        vals.append(cb["value"])
    v = statistics.median(vals)
    cb["value"] = v
    line = {"impl": "reference", "metric": "J+K Fock builds/s", "value": v, "unit": "builds/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD["name"], "nbf": bas.nbf, "cutoff": WORKLOAD["cutoff"]},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": "builds/s", "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from openqp_gb300 import build as bld
    bld.build()
    from openqp_gb300.fock import NCLASS, FockBuilder, class_flops, class_labels, fp64_peak_tflops, routec_init, \
        routec_fock_jk
    bas, d = make_workload()
    fb = FockBuilder(bas, cutoff=WORKLOAD["cutoff"])
    ntri = fb.ntri
    dt = torch.from_numpy(d[None]).cuda()
    out = torch.empty_like(dt)
    st = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed(precision, steps=None):
        steps = args.steps if steps is None else steps
        fb.set_precision(precision, args.mixed_threshold)
        for _ in range(args.warmup):
            fb.fock_jk_device(dt, out=out)
        torch.cuda.synchronize()
        times, stats = [], []
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        for _ in range(steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fb.fock_jk_device(dt, out=out, stream=st)
            e1.record(st)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            stats.append(fb.stats())
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        tsum = max_over_ranks(sum(times) / 1000.0)
        return tsum, stats, out.clone()

    mixed = None
    if args.precision != "fp64":
        t64, _, f64 = timed("fp64")
    sampler = ClockSampler(local)
    sampler.start()
    wall0 = time.perf_counter()
    tsum, stats, fval = timed(args.precision)
    wall = time.perf_counter() - wall0
    clocks = sampler.stop()
    value = ws * args.steps / tsum
    if args.precision != "fp64":
        from openqp_gb300.basis import unpack
        df = (fval - f64).cpu().numpy()[0]
        de2 = 0.5 * float(np.sum(unpack(d, bas.nbf) * unpack(df, bas.nbf)))
        mixed = {"mode": args.precision, "threshold": args.mixed_threshold, "fp64_builds_per_s": ws * args.steps / t64,
                 "speedup_vs_fp64": t64 / tsum, "max_abs_dF": float(np.abs(df).max()),
                 "dE2_Eh": de2, "f32_quartet_fraction": stats[-1]["f32_quartets"] / max(1, stats[-1]["quartets"])}
    # the same build in double-float (FP32 pairs on the FP32 pipe), error against FP64
    df_mode = None
    if args.precision == "fp64" and not args.no_df:
        tdf, _, fdf = timed("df")
        ddf = (fdf - fval).cpu().numpy()[0]
        from openqp_gb300.basis import unpack
        df_mode = {"builds_per_s": ws * args.steps / tdf, "speedup_vs_fp64": tsum / tdf,
                   "max_abs_dF_vs_fp64": float(np.abs(ddf).max()),
                   "dE2_Eh": 0.5 * float(np.sum(unpack(d, bas.nbf) * unpack(ddf, bas.nbf))),
                   "arithmetic": "double-float: unevaluated pairs of FP32 numbers (~44 bits), FP64 accumulators"}
        fb.set_precision("fp64")
    # the precision split on the same build: FP32 below the bound with FP64
    # roots ("mixed", the task's form (b)) and with double-float above it
    # ("mixed-df"); speed-up over this run's FP64 value, errors against it
    split_c2 = None
    extras = args.precision == "fp64" and not args.no_extras and args.workload == "water32_ccpvdz"
    if extras:
        from openqp_gb300.basis import unpack
        nstep = max(1, min(args.steps, 5))
        split_c2 = {}
        for mode in ("mixed", "mixed-fast", "mixed-df"):
            tm, stm, fm = timed(mode, steps=nstep)
            dfm = (fm - fval).cpu().numpy()[0]
            t32 = float(np.mean([sum(x["ms_per_class_f32"]) for x in stm]))
            split_c2[mode] = {"threshold": args.mixed_threshold, "builds_per_s": nstep / tm,
                              "speedup_vs_fp64": (tsum / args.steps) / (tm / nstep),
                              "max_abs_dF_vs_fp64": float(np.abs(dfm).max()),
                              "dE2_Eh": 0.5 * float(np.sum(unpack(d, bas.nbf) * unpack(dfm, bas.nbf))),
                              "f32_quartet_fraction": stm[-1]["f32_quartets"] / max(1, stm[-1]["quartets"]),
                              "f32_prim_quartet_fraction": stm[-1]["f32_prim_quartets"] /
                              max(1, stm[-1]["prim_quartets"]),
                              "fp64_launch_ms": float(np.mean([sum(x["ms_per_class"]) for x in stm])) - t32,
                              "fp32_launch_ms": t32}
        fb.set_precision("fp64")
    # e2e through the seam with host buffers
    e2e_t = [float("nan")]
    if not args.no_e2e:
        routec_init(bas, WORKLOAD["cutoff"])
        dflat = np.ascontiguousarray(d)
        routec_fock_jk(dflat, bas.nbf, 1)
        e2e_t = []
    for _ in range(0 if args.no_e2e else args.steps):
        t0 = time.perf_counter()
        f_host, info = routec_fock_jk(dflat, bas.nbf, 1)
        e2e_t.append(time.perf_counter() - t0)
        if info != 0:
            raise RuntimeError("routec_fock_jk returned info=%d" % info)
    e2e_sum = max_over_ranks(sum(e2e_t))
    e2e = ws * args.steps / e2e_sum
    # roofline of the dominant class kernel (mean over the timed steps)
    labels = class_labels()
    ms = np.mean([s["ms_per_class"] for s in stats], axis=0)
    cdom = int(np.argmax(ms))
    s0 = stats[-1]
    flops = class_flops(cdom, s0["prim_per_class"][cdom], s0["per_class"][cdom], nk=1, pure=bool(bas.harmonic.any()))
    achieved = flops / (ms[cdom] * 1e-3) / 1e12
    total_flops = sum(class_flops(c, s0["prim_per_class"][c], s0["per_class"][c], nk=1, pure=bool(bas.harmonic.any()))
                      for c in range(NCLASS))
    peak = fp64_peak_tflops()
    if rank == 0:
        line = {"metric": "J+K Fock builds/s", "value": value, "unit": "builds/s", "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * tsum / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded water cluster and Loewdin density)",
                "config": {"workload": WORKLOAD["name"], "nbf": bas.nbf, "nshell": int(len(bas.am)),
                           "cutoff": WORKLOAD["cutoff"], "l2": "flushed (256 MB write) before every timed step",
                           "parallelism": "replicas" if ws > 1 else "single GPU"},
                "e2e": {"value": e2e, "unit": "builds/s", "h2d_bytes_per_step": int(8 * ntri),
                        "d2h_bytes_per_step": int(8 * ntri)},
                "roofline": {"bound": "fp64", "kernel": labels[cdom], "achieved": achieved, "peak": peak,
                             "unit": "TFLOP/s", "frac": achieved / peak,
                             "traffic": WORKLOAD.get("traffic", {}).get(labels[cdom]),
                             "traffic_unit": "DRAM bytes per build of the class (ncu, scaled from a small case)",
                             "peak_source": "measured: FP64 FMA-chain probe on this device",
                             "kernel_ms": float(ms[cdom]), "build_fp64_tflops": total_flops / (tsum / args.steps) / 1e12},
                "quartets_per_s": s0["quartets"] / (tsum / args.steps),
                "prim_quartets_per_s": s0["prim_quartets"] / (tsum / args.steps),
                "gpu_launches": int(sum(s["launches"] for s in stats)),
                "wall_s": wall, "clocks": clocks,
                "class_ms": {labels[c]: round(float(ms[c]), 3) for c in range(NCLASS) if ms[c] > 0},
                "class_quartets": {labels[c]: s0["per_class"][c] for c in range(NCLASS) if s0["per_class"][c]},
                "class_prim_quartets": {labels[c]: s0["prim_per_class"][c] for c in range(NCLASS)
                                        if s0["prim_per_class"][c]},
                "list_ms": s0["list_ms"]}
        if mixed is not None:
            line["dtype"] = {"df": "f32x2 (double-float)", "mixed-df": "f32 + f32x2 (double-float)"}.get(args.precision,
                                                                                                        "f32+f64")
            line["precision_split"] = mixed
        if df_mode is not None:
            line["double_float_mode"] = df_mode
        if split_c2 is not None:
            line["precision_split_modes"] = split_c2
        if extras and ws == 1:
            line["north_star"] = north_star_extras(args, flush, st, peak)
        if not args.no_cpu:
            cb, _ = cpu_baseline(bas, d, budget_s=args.cpu_budget)
            line["cpu_baseline"] = cb
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_scf_bench(args):
    """Direct SCF with the GPU Fock build as its two-electron part (host
    buffers through the C ABI in every iteration).  With mixed_scf: the same
    SCF in plain FP64 (the reference energy) and with the precision split plus
    incremental dD builds, energy error against the FP64 run."""
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    from openqp_gb300 import build as bld
    bld.build()
    from openqp_gb300 import onee, scf, workloads
    from openqp_gb300.fock import FockBuilder
    bas, d_warm = make_workload()
    S, T, V = onee.one_electron(bas)
    H = T + V
    enuc = onee.nuclear_repulsion(bas)
    nocc = workloads.nelectrons(bas) // 2
    fb = FockBuilder(bas, cutoff=WORKLOAD["cutoff"])

    def run(precision, incremental):
        if precision == "fp64":
            fb.set_precision("fp64")
        else:
            fb.set_precision(precision, args.mixed_threshold)
        tb = []
        stats = []

        def fock2e(dp):
            t0 = time.perf_counter()
            f = fb.fock_jk(dp)
            tb.append(time.perf_counter() - t0)
            stats.append(fb.stats())
            return f

        fock2e(d_warm)   # warm-up build on the seeded density (sizes the quartet lists)
        tb.clear(); stats.clear()
        w0 = time.perf_counter()
        r = scf.run_scf(bas.nbf, S, H, enuc, nocc, nocc, fock2e, kind="rhf", conv=1e-9, maxit=60,
                        incremental=incremental)
        wall = time.perf_counter() - w0
        q = sum(s_["quartets"] for s_ in stats)
        return dict(energy=r["energy"], converged=bool(r["converged"]), iterations=r["iterations"], builds=len(tb),
                    build_s=sum(tb), wall_s=wall, builds_per_s=len(tb) / sum(tb), quartets_per_s=q / sum(tb),
                    f32_quartet_fraction=(sum(s_["f32_quartets"] for s_ in stats) / max(1, q)))

    sampler = ClockSampler(local)
    sampler.start()
    ref = run("fp64", False)
    mixed = None
    if WORKLOAD.get("mixed_scf"):
        prec = args.precision if args.precision != "fp64" else "mixed-fast"
        mixed = run(prec, True)
        mixed.update(mode=prec, threshold=args.mixed_threshold, incremental=True,
                     dE_vs_fp64_Eh=mixed["energy"] - ref["energy"],
                     speedup_build_time=ref["build_s"] / mixed["build_s"])
    clocks = sampler.stop()
    main_run = mixed if mixed else ref
    line = {"metric": "J+K Fock builds/s inside a direct SCF", "value": main_run["builds_per_s"], "unit": "builds/s",
            "n_gpus": ws, "steps": main_run["builds"], "warmup": 1,
            "ms_per_step": 1000.0 * main_run["build_s"] / main_run["builds"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if mixed else "f64",
            "data": "synthetic (seeded geometry; core-Hamiltonian guess)",
            "config": {"workload": WORKLOAD["name"], "nbf": bas.nbf, "cutoff": WORKLOAD["cutoff"],
                       "conv": "dE < 1e-9, DIIS error < 1e-6", "guess": "core Hamiltonian",
                       "l2": "not flushed: consecutive SCF iterations (inputs ~5 MB)"},
            "e2e": {"value": main_run["builds"] / main_run["wall_s"], "unit": "SCF iterations/s (wall, incl. host DIIS "
                    "and diagonalisation)", "h2d_bytes_per_step": int(8 * bas.nbf * (bas.nbf + 1) // 2),
                    "d2h_bytes_per_step": int(8 * bas.nbf * (bas.nbf + 1) // 2)},
            "scf_fp64": ref, "clocks": clocks}
    if mixed:
        line["scf_mixed_incremental"] = mixed
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_grad(args):
    """Gradient evaluations/s: the two-electron HF gradient (derivative ERIs
    contracted with the two-particle density), D resident on the host side
    of the C ABI (one H2D of the packed density and one D2H of dE/dR per
    evaluation are inside the timed call)."""
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    from openqp_gb300 import build as bld
    bld.build()
    from openqp_gb300.fock import FockBuilder, fp64_peak_tflops
    bas, d = make_workload()
    fb = FockBuilder(bas, cutoff=WORKLOAD["cutoff"])
    if WORKLOAD.get("mrsf_grad"):
        return run_grad_mrsf(args, bas, fb)
    for _ in range(args.warmup):
        fb.grad2(d)
    torch.cuda.synchronize()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    sampler = ClockSampler(local)
    sampler.start()
    times, g = [], None
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g = fb.grad2(d)
        times.append(time.perf_counter() - t0)
    clocks = sampler.stop()
    st = fb.grad_stats()
    value = ws * args.steps / sum(times)
    # the same gradient with the precision split (FP32 below the bound), error against FP64
    prec = args.precision if args.precision != "fp64" else "mixed-fast"
    fb.set_precision(prec, args.mixed_threshold)
    for _ in range(2):
        gm = fb.grad2(d)
    tm = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        gm = fb.grad2(d)
        tm.append(time.perf_counter() - t0)
    stm = fb.grad_stats()
    split = {"mode": prec, "threshold": args.mixed_threshold, "grad_evals_per_s": args.steps / sum(tm),
             "speedup_vs_fp64": sum(times) / sum(tm), "max_abs_grad_error_Eh_bohr": float(np.abs(gm - g).max()),
             "f32_quartet_fraction": stm["f32_quartets_listed"] / max(1, stm["quartets_listed"])}
    fb.set_precision("fp64")
    # the CAM gradient (grd2_driver's two-pass branch, CAM-B3LYP's alpha, beta, mu) of the same density
    fb.grad2_cam(d, 0.19, 0.46, 0.33)
    tc = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fb.grad2_cam(d, 0.19, 0.46, 0.33)
        tc.append(time.perf_counter() - t0)
    cam_line = {"alpha": 0.19, "beta": 0.46, "mu": 0.33, "grad_evals_per_s": args.steps / sum(tc)}
    line = {"metric": "two-electron gradient evaluations/s", "value": value, "unit": "grad evals/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * sum(times) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded water cluster and Loewdin density)",
            "config": {"workload": WORKLOAD["name"], "nbf": bas.nbf, "natom": bas.natom, "cutoff": WORKLOAD["cutoff"],
                       "l2": "flushed (256 MB write) before every timed step"},
            "e2e": {"value": value, "unit": "grad evals/s", "h2d_bytes_per_step": int(d.nbytes),
                    "d2h_bytes_per_step": int(8 * 3 * bas.natom)},
            "grad_stats": st, "quartets_per_s": st["quartets"] / (sum(times) / args.steps),
            "prim_quartets_per_s": st["prim_quartets"] / (sum(times) / args.steps),
            "fp64_peak_tflops": fp64_peak_tflops(), "clocks": clocks, "precision_split": split, "cam": cam_line,
            "max_abs_grad": float(np.abs(g).max()), "sum_grad": float(np.abs(g.sum(axis=0)).max())}
    if not args.no_cpu and rank == 0:
        line["cpu_baseline"] = cpu_baseline_grad(bas, d, args.cpu_budget)
    if rank == 0:
        print(json.dumps(line), flush=True)


MRSF_GRAD_ARGS = (0.5, 0.5, 1.0, (0.5, 0.5, 0.5), 1)   # hfscale, hfscale2, coulscale, spc scales, singlet


def run_grad_mrsf(args, bas, fb):
    """MRSF two-electron gradient evaluations/s through FockBuilder.grad2_mrsf
    (host matrices in, dE/dR out: the seam's own data flow, so value and e2e
    coincide), with the plain RHF-form gradient of the same total density for
    comparison."""
    import torch
    ws, rank, local = dist_env()
    from openqp_gb300 import workloads
    from openqp_gb300.basis import pack
    from openqp_gb300.fock import fp64_peak_tflops
    d, p, spc = workloads.mrsf_gradient_inputs(bas, WORKLOAD["seed"])
    for _ in range(args.warmup):
        fb.grad2_mrsf(d, p, spc, *MRSF_GRAD_ARGS)
    torch.cuda.synchronize()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    sampler = ClockSampler(local)
    sampler.start()
    times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g = fb.grad2_mrsf(d, p, spc, *MRSF_GRAD_ARGS)
        times.append(time.perf_counter() - t0)
    clocks = sampler.stop()
    st = fb.grad_stats()
    value = ws * args.steps / max_over_ranks(sum(times))
    dt = pack(d[0] + d[1])
    fb.grad2(dt)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        fb.grad2(dt)
    t_plain = (time.perf_counter() - t0) / args.steps
    nb = int(8 * (d.size + p.size + spc.size))
    line = {"metric": "MRSF two-electron gradient evaluations/s", "value": value, "unit": "grad evals/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * sum(times) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded water cluster, triplet-reference densities, seeded response densities)",
            "config": {"workload": WORKLOAD["name"], "nbf": bas.nbf, "natom": bas.natom, "cutoff": WORKLOAD["cutoff"],
                       "hfscale": MRSF_GRAD_ARGS[0], "hfscale2": MRSF_GRAD_ARGS[1],
                       "spcscale": list(MRSF_GRAD_ARGS[3]), "kind": "singlet",
                       "l2": "flushed (256 MB write) before every timed step"},
            "e2e": {"value": value, "unit": "grad evals/s", "h2d_bytes_per_step": nb,
                    "d2h_bytes_per_step": int(8 * 3 * bas.natom)},
            "grad_stats": st, "quartets_per_s": st["quartets"] / (sum(times) / args.steps),
            "prim_quartets_per_s": st["prim_quartets"] / (sum(times) / args.steps),
            "plain_rhf_form_grad_evals_per_s": 1.0 / t_plain,
            "fp64_peak_tflops": fp64_peak_tflops(), "clocks": clocks,
            "max_abs_grad": float(np.abs(g).max()), "sum_grad": float(np.abs(g.sum(axis=0)).max())}
    if not args.no_cpu and rank == 0:
        line["cpu_baseline"] = cpu_baseline_grad_mrsf(bas, d, p, spc, args.cpu_budget)
    if rank == 0:
        print(json.dumps(line), flush=True)


def cpu_baseline_grad_mrsf(bas, d, p, spc, budget_s):
    """The oracle's grd2 restatement with the MRSF density (all host cores) on
    1/stride of the bra shell pairs, scaled by stride."""
    from oracle import oracle
    oracle.build()
    o = oracle.Oracle(bas, cutoff=WORKLOAD["cutoff"])
    cores = os.cpu_count()

    def run(stride, offset):
        t0 = time.perf_counter()
        o.grad2e_mrsf(d, p, spc, *MRSF_GRAD_ARGS, nthreads=cores, stride=stride, offset=offset)
        return time.perf_counter() - t0, None

    t, stride, _ = sampled(run, budget_s)
    return {"value": 1.0 / t, "unit": "grad evals/s", "cores": cores, "kind": "port", "engine": ENGINE_GRAD,
            "sample": "oracle grd2 restatement with the MRSF two-particle density over 1/%d of the bra shell pairs "
                      "(the middle pair of every %d), x%d; %d quartets in the sample"
                      % (stride, stride, stride, o.last_grad2e_quartets)}


def cpu_baseline_grad(bas, d, budget_s):
    """The oracle's grd2 restatement (all host cores) on 1/stride of the bra
    shell pairs, scaled by stride."""
    from openqp_gb300.basis import unpack
    from oracle import oracle
    oracle.build()
    o = oracle.Oracle(bas, cutoff=WORKLOAD["cutoff"])
    D = unpack(d, bas.nbf)
    cores = os.cpu_count()

    def run(stride, offset):
        t0 = time.perf_counter()
        o.grad2e(D, nthreads=cores, stride=stride, offset=offset)
        return time.perf_counter() - t0, None

    t, stride, _ = sampled(run, budget_s)
    return {"value": 1.0 / t, "unit": "grad evals/s", "cores": cores, "kind": "port", "engine": ENGINE_GRAD,
            "sample": "oracle grd2 restatement (McMurchie-Davidson derivative integrals) over 1/%d of the bra shell "
                      "pairs (the middle pair of every %d), x%d; %d quartets in the sample"
                      % (stride, stride, stride, o.last_grad2e_quartets)}


def pct(v, q):
    return float(np.percentile(np.asarray(v), q))


def named_workload(name):
    """Basis and density of another workload of the table (the current
    workload is restored afterwards)."""
    saved = dict(WORKLOAD)
    try:
        WORKLOAD.clear()
        WORKLOAD.update(WORKLOADS[name])
        return make_workload()
    finally:
        WORKLOAD.clear()
        WORKLOAD.update(saved)


def event_times(fn, steps, flush, st):
    """CUDA-event durations (ms) of fn(stream) on st, L2 flushed before each."""
    import torch
    times = []
    for _ in range(steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        fn(st)
        e1.record(st)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    return times


def graph_replays(bb, d, out, precision, threshold, steps, warmup, flush, st):
    """Event-timed replays of a context's captured graph in one precision
    mode: (times in ms, a copy of the output, build statistics)."""
    import torch
    if precision == "fp64":
        bb.set_precision("fp64")
    else:
        bb.set_precision(precision, threshold)
    for _ in range(max(warmup, 2)):
        bb.fock_jk_graph(d, out=out, stream=st)
    torch.cuda.synchronize()
    times = event_times(lambda s: bb.fock_jk_graph(d, out=out, stream=s), steps, flush, st)
    return times, out.clone(), bb.stats()


def binned_latency(bases, dens, cutoff, nbins, steps, warmup, flush, st, precision="fp64", threshold=1e-6):
    """Per-molecule completion latency of a batch served as size-ordered
    sub-batches: the molecules sorted by basis size and split into nbins
    sub-batches of equal molecule count, each its own context with its own
    captured graph, replayed in order on one stream with an event after each.
    A molecule's latency is the time from the start of the sequence to its
    sub-batch's event (its Fock matrix is final then).  Returns (latencies in
    ms, one per molecule and step; aggregate builds/s of the sequence)."""
    import torch
    from openqp_gb300.fock import BatchFockBuilder
    order = np.argsort([b.nbf for b in bases], kind="stable")
    subs = []
    for g in np.array_split(order, nbins):
        bb = BatchFockBuilder([bases[i] for i in g], cutoff=cutoff)
        if precision != "fp64":
            bb.set_precision(precision, threshold)
        d = torch.from_numpy(bb.pack([dens[i] for i in g])[None]).cuda()
        subs.append((bb, d, torch.empty_like(d), len(g)))
    for _ in range(max(warmup, 2)):
        for bb, d, out, _ in subs:
            bb.fock_jk_graph(d, out=out, stream=st)
    torch.cuda.synchronize()
    lat, total = [], 0.0
    for _ in range(steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        evs = []
        for bb, d, out, n in subs:
            bb.fock_jk_graph(d, out=out, stream=st)
            e = torch.cuda.Event(enable_timing=True)
            e.record(st)
            evs.append((e, n))
        evs[-1][0].synchronize()
        for e, n in evs:
            lat.extend([e0.elapsed_time(e)] * n)
        total += e0.elapsed_time(evs[-1][0])
    for bb, _, _, _ in subs:
        bb.close()
    return lat, len(bases) * steps / (total / 1000.0)


def north_star_extras(args, flush, st, peak):
    """The rest of the task's metric beside the headline plain-FP64 build, in
    the same process (one GPU): the batched builds of the 256 water clusters
    (FP64, mixed and mixed-df graphs of the same batching, per-molecule
    latency), the (H2O)16 6-31G(d) two-electron gradient in FP64 and with the
    precision split, and the (dd|dd) fraction of the FP64 peak."""
    import torch
    from openqp_gb300 import workloads
    from openqp_gb300.basis import unpack
    from openqp_gb300.fock import BatchFockBuilder, FockBuilder, class_flops, class_labels
    nstep = max(1, min(args.steps, 5))
    thr = args.mixed_threshold
    res = {}
    # --- 256 water clusters, 6-31G, one captured graph (built-in launch defaults)
    sizes, bases, dens = workloads.water_batch(256, 0, basis="6-31g")
    bb = BatchFockBuilder(bases, cutoff=1e-10)
    d = torch.from_numpy(bb.pack(dens)[None]).cuda()
    out = torch.empty_like(d)
    rate = {}
    t64, f64, _ = graph_replays(bb, d, out, "fp64", thr, nstep, args.warmup, flush, st)
    rate["fp64"] = 256 * nstep / (sum(t64) / 1000.0)
    f64n = f64.cpu().numpy()[0]
    batch = {"workload": "256 water clusters (1-16 H2O, uniform, seed 0), 6-31G, one captured graph per mode",
             "steps": nstep, "fp64_graph_builds_per_s": rate["fp64"]}
    def max_de2(fmn):
        de = 0.0
        for m, bas in enumerate(bases):
            o, n = bb.tri0[m], bas.nbf
            t = n * (n + 1) // 2
            de = max(de, abs(0.5 * float(np.sum(unpack(dens[m], n) * unpack(fmn[o:o + t] - f64n[o:o + t], n)))))
        return de

    def launch_split():
        # one direct (event-timed) build in the current mode: class time in FP64 and FP32 launches
        bb.fock_jk_device(d, out=out, stream=st)
        s0 = bb.stats()
        t32 = float(sum(s0["ms_per_class_f32"]))
        return {"fp64_launch_ms": float(sum(s0["ms_per_class"])) - t32, "fp32_launch_ms": t32,
                "f32_prim_quartet_fraction": s0["f32_prim_quartets"] / max(1, s0["prim_quartets"])}

    batch["fp64_launch_split"] = launch_split()
    for mode in ("mixed", "mixed-fast", "mixed-df"):
        tm, fm, stm = graph_replays(bb, d, out, mode, thr, nstep, args.warmup, flush, st)
        fmn = fm.cpu().numpy()[0]
        r = 256 * nstep / (sum(tm) / 1000.0)
        batch[mode] = {"graph_builds_per_s": r, "speedup_vs_fp64_graph": r / rate["fp64"], "threshold": thr,
                       "max_abs_dF_vs_fp64": float(np.abs(fmn - f64n).max()), "max_abs_dE2_Eh": max_de2(fmn),
                       "f32_quartet_fraction": stm["f32_quartets"] / max(1, stm["quartets"]),
                       "launch_split": launch_split()}
    # the split threshold against the energy error (graph rates, 2 replays per point)
    sweep = []
    for mode in ("mixed", "mixed-df"):
        for t in (1e-7, 1e-6, 1e-5, 1e-4, 1e-3):
            tm, fm, stm = graph_replays(bb, d, out, mode, t, 2, 1, flush, st)
            r = 256 * 2 / (sum(tm) / 1000.0)
            sweep.append({"mode": mode, "threshold": t, "speedup_vs_fp64_graph": r / rate["fp64"],
                          "max_abs_dE2_Eh": max_de2(fm.cpu().numpy()[0]),
                          "f32_quartet_fraction": stm["f32_quartets"] / max(1, stm["quartets"])})
    batch["threshold_sweep"] = sweep
    bb.set_precision("fp64")
    bb.close()
    lat, rate_b = binned_latency(bases, dens, 1e-10, 8, nstep, args.warmup, flush, st)
    batch["per_molecule_latency_fp64"] = {
        "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99), "aggregate_builds_per_s": rate_b,
        "how": "molecules sorted by size into 8 sub-batches of 32, one captured graph each, replayed in order; "
               "latency = start of the sequence to the event after the molecule's sub-batch"}
    res["batch256_631g"] = batch
    # --- two-electron gradient of (H2O)16 6-31G(d), host matrices in and out (FockBuilder.grad2)
    gbas, gd = named_workload("grad_water16_631gd")
    gfb = FockBuilder(gbas, cutoff=1e-10)
    grad = {"workload": WORKLOADS["grad_water16_631gd"]["name"], "steps": nstep}
    g64 = None
    for mode in ("fp64", "mixed", "mixed-fast"):
        if mode == "fp64":
            gfb.set_precision("fp64")
        else:
            gfb.set_precision(mode, thr)
        for _ in range(2):
            g = gfb.grad2(gd)
        ts = []
        for _ in range(nstep):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            g = gfb.grad2(gd)
            ts.append(time.perf_counter() - t0)
        r = nstep / sum(ts)
        if mode == "fp64":
            g64, r64 = g, r
            grad["fp64_grad_evals_per_s"] = r
        else:
            grad[mode] = {"grad_evals_per_s": r, "speedup_vs_fp64": r / r64, "threshold": thr,
                          "max_abs_grad_error_Eh_bohr": float(np.abs(g - g64).max())}
    gfb.close()
    res["grad_water16_631gd"] = grad
    # --- (dd|dd) only: 64 Cartesian d shells on a lattice
    dbas, dd = named_workload("dd_only")
    dfb = FockBuilder(dbas, cutoff=1e-10)
    ddt = torch.from_numpy(dd[None]).cuda()
    dout = torch.empty_like(ddt)
    for _ in range(2):
        dfb.fock_jk_device(ddt, out=dout)
    ms = []
    for _ in range(nstep):
        flush.zero_()
        dfb.fock_jk_device(ddt, out=dout, stream=st)
        ms.append(dfb.stats()["ms_per_class"][20])
    s0 = dfb.stats()
    assert class_labels()[20] == "(dd|dd)"
    fl = class_flops(20, s0["prim_per_class"][20], s0["per_class"][20], nk=1, pure=False)
    tf = fl / (float(np.mean(ms)) * 1e-3) / 1e12
    res["dd_dd_lattice"] = {"workload": WORKLOADS["dd_only"]["name"], "kernel_ms": float(np.mean(ms)),
                            "achieved_tflops": tf, "fp64_peak_tflops": peak, "frac_of_fp64_peak": tf / peak}
    dfb.close()
    return res


def run_batch(args):
    """Batched builds: one context over all clusters, replayed from one CUDA
    graph, against the plain FP64 path building each cluster on its own."""
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from openqp_gb300 import build as bld
    bld.build()
    from openqp_gb300 import autotune, workloads
    from openqp_gb300.basis import unpack
    from openqp_gb300.fock import NCLASS, BatchFockBuilder, FockBuilder, class_flops, class_labels, fp64_peak_tflops
    sizes, bases, dens = workloads.water_batch(WORKLOAD["batch"], WORKLOAD["seed"] + rank, basis=WORKLOAD["basis"])
    nmol = len(bases)
    st = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    # --- plain FP64 path, one cluster per build (device-resident densities)
    singles = [FockBuilder(b, cutoff=WORKLOAD["cutoff"]) for b in bases]
    dts = [torch.from_numpy(d[None]).cuda() for d in dens]
    outs = [torch.empty_like(x) for x in dts]
    for _ in range(args.warmup):
        for fb, x, o in zip(singles, dts, outs):
            fb.fock_jk_device(x, out=o)
    torch.cuda.synchronize()
    lat1 = []
    t_single = 0.0
    for _ in range(args.steps):
        flush.zero_()
        for fb, x, o in zip(singles, dts, outs):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fb.fock_jk_device(x, out=o, stream=st)
            e1.record(st)
            e1.synchronize()
            lat1.append(e0.elapsed_time(e1))
    t_single = sum(lat1) / 1000.0
    plain_rate = nmol * args.steps / t_single
    f_single = [o.clone() for o in outs]
    del singles
    # --- batched context, tuned per class, replayed from its graph
    bb = BatchFockBuilder(bases, cutoff=WORKLOAD["cutoff"])
    dflat = bb.pack(dens)
    d = torch.from_numpy(dflat[None]).cuda()
    out = torch.empty_like(d)
    tune = autotune.autotune(bb, d, "batch%d-%s-seed%d" % (nmol, WORKLOAD["basis"], WORKLOAD["seed"]), reps=1)

    def replay(precision):
        if precision == "fp64":
            bb.set_precision("fp64")
        else:
            bb.set_precision(precision, args.mixed_threshold)
        for _ in range(max(args.warmup, 2)):
            bb.fock_jk_graph(d, out=out)
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        times = []
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            bb.fock_jk_graph(d, out=out, stream=st)
            e1.record(st)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        torch.cuda.synchronize()
        tsum = max_over_ranks(sum(times) / 1000.0)
        return tsum, times, out.clone(), bb.stats(), bb.graph_info()

    t64, times64, f64, st64, gi64 = replay("fp64")
    tdf, timesdf, fdf, _, _ = replay("df")
    tmd, timesmd, fmd, stmd, _ = replay("mixed-df")
    prec = args.precision if args.precision != "fp64" else "mixed-fast"
    sampler = ClockSampler(local)
    sampler.start()
    wall0 = time.perf_counter()
    tm, timesm, fm, stm, gim = replay(prec)
    wall = time.perf_counter() - wall0
    clocks = sampler.stop()
    value = ws * nmol * args.steps / tm
    # errors of the batched builds against the single FP64 builds, per molecule
    f64n, fmn = f64.cpu().numpy()[0], fm.cpu().numpy()[0]
    de_max, df_max, d64_max = 0.0, 0.0, 0.0
    for m, bas in enumerate(bases):
        o, n = bb.tri0[m], bas.nbf
        t = n * (n + 1) // 2
        ref = f_single[m].cpu().numpy()[0]
        d64_max = max(d64_max, float(np.abs(f64n[o:o + t] - ref).max()))
        dfm = fmn[o:o + t] - ref
        df_max = max(df_max, float(np.abs(dfm).max()))
        de_max = max(de_max, abs(0.5 * float(np.sum(unpack(dens[m], n) * unpack(dfm, n)))))
    # e2e through the batch seam with host buffers (H2D + graph + D2H per step)
    e2e = None
    if not args.no_e2e:
        from openqp_gb300._lib import lib, ptr, _i
        from openqp_gb300.fock import _batch_arrays
        nsh, nat, k = _batch_arrays(bases)
        rc = lib().routec_fock_init_batch(nmol, ptr(nsh, _i), ptr(nat, _i), ptr(k[0], _i), ptr(k[1], _i),
                                          ptr(k[2], _i), ptr(k[3]), ptr(k[4]), ptr(k[5], _i), ptr(k[6]),
                                          WORKLOAD["cutoff"])
        if rc != 0:
            raise RuntimeError("routec_fock_init_batch returned %d" % rc)
        lib().routec_fock_set_precision({"mixed": 1, "mixed-fast": 2, "df": 3, "mixed-df": 4}[prec],
                                        args.mixed_threshold)
        fh = np.zeros_like(dflat)
        info = ctypes.c_int(1)
        nm, nf = ctypes.c_int(nmol), ctypes.c_int(1)
        se, sc = ctypes.c_double(1.0), ctypes.c_double(1.0)
        for _ in range(max(args.warmup, 2)):
            lib().routec_fock_jk_batch(ptr(dflat), ptr(fh), ctypes.byref(nm), ctypes.byref(nf), ctypes.byref(se),
                                       ctypes.byref(sc), ctypes.byref(info))
        t0 = time.perf_counter()
        for _ in range(args.steps):
            lib().routec_fock_jk_batch(ptr(dflat), ptr(fh), ctypes.byref(nm), ctypes.byref(nf), ctypes.byref(se),
                                       ctypes.byref(sc), ctypes.byref(info))
            if info.value != 0:
                raise RuntimeError("routec_fock_jk_batch returned info=%d" % info.value)
        e2e_t = time.perf_counter() - t0
        lib().routec_fock_finalize()
        e2e = {"value": ws * nmol * args.steps / e2e_t, "unit": "builds/s", "h2d_bytes_per_step": int(dflat.nbytes),
               "d2h_bytes_per_step": int(dflat.nbytes)}
    # per-molecule completion latency: size-ordered sub-batches, one graph each
    lat_b, rate_b = binned_latency(bases, dens, WORKLOAD["cutoff"], 8, args.steps, args.warmup, flush, st,
                                   precision=prec, threshold=args.mixed_threshold)
    # roofline of the dominant class from a direct (event-timed) build in the same precision
    bb.fock_jk_device(d, out=out)
    s0 = bb.stats()
    labels = class_labels()
    ms = np.array(s0["ms_per_class"])
    cdom = int(np.argmax(ms))
    flops = class_flops(cdom, s0["prim_per_class"][cdom], s0["per_class"][cdom], nk=1, pure=False)
    achieved = flops / (ms[cdom] * 1e-3) / 1e12
    peak = fp64_peak_tflops()
    if rank == 0:
        line = {"metric": "J+K Fock builds/s (molecule builds, batched)", "value": value, "unit": "builds/s",
                "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * tm / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
                "data": "synthetic (seeded water clusters, Loewdin random densities)",
                "config": {"workload": WORKLOAD["name"], "nmol": nmol, "waters": {"min": min(sizes), "max": max(sizes),
                           "mean": float(np.mean(sizes))}, "nbf_total": bb.nbf, "basis": WORKLOAD["basis"],
                           "cutoff": WORKLOAD["cutoff"], "precision": prec, "mixed_threshold": args.mixed_threshold,
                           "l2": "flushed (256 MB write) before every timed step",
                           "parallelism": "replicas" if ws > 1 else "single GPU"},
                "e2e": e2e,
                "plain_fp64_unbatched": {"builds_per_s": plain_rate, "latency_ms_p50": pct(lat1, 50),
                                         "latency_ms_p99": pct(lat1, 99)},
                "batched_fp64_graph": {"builds_per_s": ws * nmol * args.steps / t64,
                                       "replay_ms_p50": pct(times64, 50), "replay_ms_p99": pct(times64, 99),
                                       "max_abs_dF_vs_single": d64_max},
                "batched_mixed_graph": {"builds_per_s": value, "replay_ms_p50": pct(timesm, 50),
                                        "replay_ms_p99": pct(timesm, 99), "max_abs_dF_vs_fp64": df_max,
                                        "max_abs_dE2_Eh": de_max,
                                        "f32_quartet_fraction": stm["f32_quartets"] / max(1, stm["quartets"])},
                "batched_double_float_graph": {"builds_per_s": ws * nmol * args.steps / tdf,
                                               "replay_ms_p50": pct(timesdf, 50),
                                               "max_abs_dF_vs_fp64": float(np.abs((fdf - f64).cpu().numpy()).max())},
                "batched_mixed_df_graph": {"builds_per_s": ws * nmol * args.steps / tmd,
                                           "replay_ms_p50": pct(timesmd, 50),
                                           "max_abs_dF_vs_fp64": float(np.abs((fmd - f64).cpu().numpy()).max()),
                                           "f32_quartet_fraction": stmd["f32_quartets"] / max(1, stmd["quartets"])},
                "speedup_vs_plain_fp64": value / plain_rate,
                "per_molecule_latency_ms": {"p50": pct(lat_b, 50), "p99": pct(lat_b, 99),
                                            "aggregate_builds_per_s": rate_b, "precision": prec,
                                            "how": "molecules sorted by size into 8 sub-batches of equal count, "
                                                   "one captured graph each, replayed in order on one stream; "
                                                   "latency = start of the sequence to the event after the "
                                                   "molecule's sub-batch"},
                "roofline": {"bound": "fp64", "kernel": labels[cdom], "achieved": achieved, "peak": peak,
                             "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                             "peak_source": "measured: FP64 FMA-chain probe on this device",
                             "kernel_ms": float(ms[cdom])},
                "autotune": {"family": tune.get("family"), "split_log2": tune["split_log2"], "chunk": tune["chunk"],
                             "ctas_per_sm": tune["ctas_per_sm"], "class_ms_sum_tuned": float(sum(tune["class_ms"])),
                             "class_ms_sum_default": float(sum(tune.get("default_class_ms", tune["class_ms"])))},
                "gpu_launches": int(gim["kernels"]) * args.steps,
                "graph": gim, "wall_s": wall, "clocks": clocks}
        if not args.no_cpu:
            line["cpu_baseline"] = cpu_baseline_batch(bases, dens, args.cpu_budget)
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def cpu_baseline_batch(bases, dens, budget_s):
    """The oracle (all host cores) building the clusters one by one, in order,
    until the budget is spent; builds/s over the clusters it finished."""
    from oracle import oracle
    oracle.build()
    cores = os.cpu_count()
    t_all, done, nbf = 0.0, 0, 0
    for bas, d in zip(bases, dens):
        o = oracle.Oracle(bas, cutoff=WORKLOAD["cutoff"])
        t0 = time.perf_counter()
        q = o.schwarz(nthreads=cores)
        o.fock_jk(d, nthreads=cores, schwarz=q)
        t_all += time.perf_counter() - t0
        done += 1
        nbf += bas.nbf
        if t_all > budget_s:
            break
    return dict(value=done / t_all, unit="builds/s", cores=cores, kind="port", engine=ENGINE_FOCK,
                sample="oracle fock_jk (with its Schwarz set-up) on the first %d of %d clusters (%d bf in all)"
                       % (done, len(bases), nbf))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=20.0, help="seconds of CPU work for the baseline sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="water32_ccpvdz", choices=sorted(WORKLOADS))
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer seam timing (profiling runs)")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed", "mixed-fast", "df", "mixed-df"])
    ap.add_argument("--mixed-threshold", type=float, default=1e-6)
    ap.add_argument("--no-df", action="store_true", help="skip the double-float comparison of the default run")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the precision-split, batch, gradient and (dd|dd) measurements of the default run")
    args = ap.parse_args()
    WORKLOAD.clear()
    WORKLOAD.update(WORKLOADS[args.workload])
    if args.impl == "reference":
        run_reference(args)
    elif "batch" in WORKLOAD:
        run_batch(args)
    elif WORKLOAD.get("grad"):
        run_grad(args)
    elif WORKLOAD.get("sigma"):
        run_sigma(args)
    elif WORKLOAD.get("td"):
        run_td(args)
    elif WORKLOAD.get("cam"):
        run_cam(args)
    elif WORKLOAD.get("scf"):
        run_scf_bench(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
