"""Benchmark: std-linear prism integrate + assemble on GB300.

Workload: Poisson -div(k grad u) = 1 on the unit cube, 100^3 hexahedra split
into 2,000,000 linear prisms (1,030,301 DOFs, 21,250,901 CRS nonzeros), node
coordinates jittered by U(+-0.2h) (seeded), k ~ lognormal(0,1) per element
(seeded), penalty Dirichlet faces on the whole boundary (80,000 faces).
A step is one integrate + assemble of all elements and boundary faces into
the CRS matrix and rhs.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).  `value` is device-resident throughput
(elements/s, CUDA events on the library's stream); `e2e` is the same metric
through the pdr_create_assemble_stiff_mat drop-in with host buffers, the
step's inputs (node coordinates, k) uploaded from and the CRS values and rhs
downloaded to page-locked host memory inside the timed region.
`--impl reference` times the CPU path (the C restatement in oracle/, all
host cores, colour-parallel as the reference's OpenMP loop) on the same
workload.
"""
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
# the whole measurement record (the printed line carries its summary)
DETAIL_FILE = os.path.abspath(os.environ.get("BENCH_DETAIL", os.path.join(ROOT, "bench_detail.json")))
sys.path.insert(0, ROOT)

METRIC = "elem/s integrate+assemble vs plain FP64 GPU @1e-10 rel; served p50/p99 latency"
UNIT = "elem/s"
N_HEX = 100
JITTER, SEED = 0.2, 1
# FP64 work per std prism.  Textbook count of the reference algorithm:
# nq*(151 + 18*ns + 2*ns) + 2*3*nq*ns^2 with nq = ns = 6.  The kernel's
# quadrature-aggregated formulation executes 289 DFMA + 213 other FP64
# instructions per element (ncu instruction mix, profiles/std_prism_elements_2M.md),
# i.e. 791 flop and 502 FP64-pipe issue slots.
TEXTBOOK_FLOP_PER_ELEM = 6 * (151 + 18 * 6 + 2 * 6) + 2 * 3 * 6 * 36
# Algorithmic DRAM bytes per element of the 100^3 x 2 workload: connectivity
# 24 + k 8 + coordinates 24 nno/nel + CRS values written once 8 nnz/nel +
# rhs 8 ndof/nel + the 42-entry int32 assembly table 168 (302 B in all)
ALG_BYTES_PER_ELEM = 24 + 8 + 24 * 1030301 / 2e6 + 8 * 21250901 / 2e6 + 8 * 1030301 / 2e6 + 4 * 42
FLOP_PER_ELEM = 2 * 289 + 213
FP64_SLOTS_PER_ELEM = 289 + 213


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--n", type=int, default=N_HEX, help=argparse.SUPPRESS)
    p.add_argument("--profile", choices=["dg", "dg_tc", "dg_tcf", "dg_dwf", "dg_dw", "dg_best", "batch", "std", "std_dw",
                                         "std_solve", "std_prep"], default=None,
                   help="small cases for ncu captures: DG p=3 anisotropic (n^3 x 2 prisms, --n), 3 assemblies "
                        "(FP64, tensor-core volume, tensor-core volume and faces, FP64 volume and double-word faces, or "
                        "double-word volume and faces) and one "
                        "block residual; or the mixed batch "
                        "(40,000 prisms + 30,000 tetrahedra, p 1..4), 3 runs; or the std prism assembly "
                        "(FP64 or double-word element arithmetic, n^3 x 2 prisms), 3 assemblies; or "
                        "the std GMRES(30) (one restart cycle, device-resident, SELL SpMV); or a served std "
                        "request's preparation (device structure build and gather scatter, 3 times)")
    return p.parse_args()


def run_profile_case(args):
    """One small case for an ncu capture of the DG kernels (volume, faces,
    block SpMV); prints its CUDA-event timings."""
    import modfem_gb300 as gb
    from modfem_gb300.mesh import anisotropic_tensors, prism_faces, structured_prism_mesh
    if args.profile in ("std", "std_dw"):
        m, k = make_problem(args.n)
        c = gb.Context(0)
        c.set_mesh(m)
        c.set_coefficients(k=k, f=1.0, g=0.0, penalty=1e7)
        c.build_structure()
        c.set_option(gb.OPT_STD_ARITH, gb.STD_DWORD if args.profile == "std_dw" else gb.STD_FP64)
        ms = []
        for _ in range(3):
            c.assemble(gb.SCATTER_ATOMIC)
            ms.append(c.last_timing()[:2])
        print(json.dumps({"profile_case": args.profile, "elements": m.nel, "timing_ms": ms}))
        c.close()
        return
    if args.profile == "std_prep":
        # a served request's std preparation: device structure build, then
        # the gather scatter (incidence on its first call), 3 times
        m, k = make_problem(args.n)
        c = gb.Context(0)
        c.set_mesh(m)
        c.set_coefficients(k=k, f=1.0, g=0.0, penalty=1e7)
        ms = []
        for _ in range(3):
            t0 = time.perf_counter()
            c.build_structure_device()
            t1 = time.perf_counter()
            c.assemble(gb.SCATTER_GATHER)
            t2 = time.perf_counter()
            ms.append([round(1e3 * (t1 - t0), 3), round(1e3 * (t2 - t1), 3)])
        print(json.dumps({"profile_case": args.profile, "elements": m.nel, "host_ms_build_assemble": ms}))
        c.close()
        return
    if args.profile == "std_solve":
        m, k = make_problem(args.n)
        c = gb.Context(0)
        c.set_mesh(m)
        c.set_coefficients(k=k, f=1.0, g=0.0, penalty=1e7)
        nd, nnz, _ = c.build_structure()
        c.assemble(gb.SCATTER_ATOMIC)
        _, it, _, _ = c.solve(30, 30, 1e-14)
        t = c.last_solve_timing()
        print(json.dumps({"profile_case": args.profile, "dofs": nd, "nnz": nnz, "iterations": it,
                          "solve_ms": t[0], "spmv_ms": t[1] / max(t[2], 1),
                          "spmv_gbs": (12 * nnz + 16 * nd) / (t[1] / max(t[2], 1) * 1e-3) / 1e9}))
        c.close()
        return
    if args.profile == "batch":
        from modfem_gb300.mesh import lognormal_k, structured_tet_mesh
        NP, NT = 40_000, 30_000
        m, t = structured_prism_mesh(28, jitter=JITTER, seed=SEED), structured_tet_mesh(18, jitter=JITTER, seed=SEED)
        rng = np.random.default_rng(SEED)
        pp, tp = rng.integers(1, 5, NP), rng.integers(1, 5, NT)
        A = lognormal_k(NP + NT, seed=SEED)[:, None] * np.eye(3).reshape(1, 9)
        b = gb.Batch(0)
        b.set(m.coords[m.el_nodes[:NP]], A[:NP], pp, t.coords[t.el_nodes[:NT]], A[NP:], tp)
        b.set_variants([0, 0, 0, 2, 1], [0, 4, 4, 4, 1])
        ms = [b.run() for _ in range(3)]
        print(json.dumps({"profile_case": "batch", "elements": NP + NT, "timing_ms": ms}))
        b.close()
        return
    m = structured_prism_mesh(args.n, jitter=JITTER, seed=SEED)
    c = gb.Context(0)
    c.set_mesh(m)
    c.set_coefficients(D=anisotropic_tensors(m.nel, seed=SEED), f=1.0, g=0.0)
    c.dg_set_degrees(np.full(m.nel, 3))
    c.dg_set_faces(prism_faces(m), penalty=10.0)
    c.dg_build_structure()
    c.dg_set_volume_kernel({"dg_tc": gb.DG_VOLUME_TC, "dg_tcf": gb.DG_VOLUME_TC, "dg_dw": gb.DG_VOLUME_DWORD,
                            "dg_best": gb.DG_VOLUME_DWORD}.get(args.profile, gb.DG_VOLUME_FP64))
    c.dg_set_face_kernel({"dg_tcf": gb.DG_FACE_TC, "dg_dwf": gb.DG_FACE_DWORD, "dg_dw": gb.DG_FACE_DWORD,
                          "dg_best": gb.DG_FACE_TC_DWORD}.get(args.profile, gb.DG_FACE_FP64))
    for _ in range(3):
        c.dg_assemble()
    r = c.dg_compute_residual(np.zeros(c.dg_ndof))
    print(json.dumps({"profile_case": args.profile, "elements": m.nel, "timing_ms": c.dg_last_timing()[:3],
                      "residual_max": float(np.abs(r).max())}))
    c.close()


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl"
        try:
            import torch
            if not torch.cuda.is_available():
                backend = "gloo"
            else:
                torch.cuda.set_device(local)
        except Exception:
            backend = "gloo"
        dist.init_process_group(backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, ws):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(s[1]) for s in self.samples if len(s) >= 9 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) >= 9 and s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples if len(s) >= 9 for i in range(4)
                          if s[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def read_profile_traffic():
    """DRAM bytes per element-kernel launch from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "std_prism_elements_2M.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.strip().startswith("dram_bytes_per_launch"):
            try:
                return int(line.split("=")[1].split()[0])
            except Exception:
                return None
    return None


def hbm_peak_gbs():
    """Measured copy bandwidth of the GB300s (MEASURED_PEAKS.json),
    or None when the file is absent."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"])
    except (OSError, ValueError, KeyError, TypeError):
        return None


def source_digest(names):
    """sha256 (first 16 hex digits) over the named kernel sources under
    modfem_gb300/csrc, in order: ties a committed ncu summary to the code it
    measured."""
    import hashlib
    h = hashlib.sha256()
    for n in names:
        with open(os.path.join(ROOT, "modfem_gb300", "csrc", n), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


# sources of the std element kernels (the ncu summaries carry their digest)
STD_KERNEL_SOURCES = ("std_kernels.cu", "prism_std.cuh", "prism_dw.cuh", "dword.cuh")


def read_profile_values(name):
    """``key = number`` lines of a committed ncu summary under profiles/."""
    out = {}
    p = os.path.join(ROOT, "profiles", name)
    if os.path.exists(p):
        for line in open(p):
            parts = line.strip().split("=")
            if len(parts) >= 2 and parts[0].strip().replace("_", "").isalnum() and " " not in parts[0].strip():
                try:
                    out[parts[0].strip()] = float(parts[1].split()[0])
                except (ValueError, IndexError):
                    if parts[0].strip() == "source_sha256" and parts[1].split():
                        out["source_sha256"] = parts[1].split()[0]
    return out


def sm_count(device):
    try:
        import torch
        return torch.cuda.get_device_properties(device).multi_processor_count
    except Exception:
        return 152


def make_problem(n):
    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh
    m = structured_prism_mesh(n, jitter=JITTER, seed=SEED)
    k = lognormal_k(m.nel, seed=SEED)
    return m, k


def cpu_assemble(m, k, nthreads, reps=1):
    """The C restatement's colour-parallel integrate + assemble; seconds per run."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    d, nd = O.dof_order(m.el_nodes, m.nno)
    rp, ci = O.crs_structure(m.el_nodes, d, nd)
    col, nc = O.color_entities(d[m.el_nodes], nd)
    perm = np.argsort(col, kind="stable").astype(np.int32)
    cptr = np.zeros(nc + 1, np.int32)
    cptr[1:] = np.cumsum(np.bincount(col, minlength=nc))
    times = []
    for _ in range(reps):
        val, rhs, t = O.std_prism_assemble(m, k, d, rp, ci, color_ptr=cptr, perm=perm, nthreads=nthreads)
        times.append(t)
    return times, val, rhs


def dg_fma_per_element(p):
    """FP64 FMAs of the DG volume kernel per element: nq (9 ns + 3 ns (ns+1)/2)."""
    ns = {1: 6, 2: 18, 3: 40, 4: 75}[p]
    nq = {1: 6, 2: 18, 3: 48, 4: 80}[p]
    return nq * (9 * ns + 3 * ns * (ns + 1) // 2)


DG_NQF = {1: (3, 4), 2: (6, 9), 3: (12, 16), 4: (16, 25)}  # face rule points (triangle, quad)


def dg_face_fma(F, pdeg):
    """FP64 FMAs of the face block products: every face contributes its full
    (ns1+ns2)^2 matrix (both owners' rows) at 2 FMA per entry and point."""
    ns = np.array([0, 6, 18, 40, 75])
    p1 = pdeg[F.el1]
    p2 = np.where(F.el2 >= 0, pdeg[np.maximum(F.el2, 0)], 0)
    pr = np.maximum(p1, p2)
    nq = np.array([DG_NQF[int(a)][int(b)] for a, b in zip(pr, (F.type == 4).astype(int))])
    return float(np.sum(2.0 * nq * (ns[p1] + ns[p2]).astype(float) ** 2))


def bench_dg(gb, local, steps, fp64_peak, gmres_iters=100):
    """The DG prism system: 60^3 x 2 = 432,000 p=3 prisms with the
    anisotropic tensor R diag(1, 0.1, 0.01) R^T, and 58^3 x 2 = 390,224 prisms
    with p drawn uniformly from 1..4 and lognormal k.  A step integrates every
    element (volume kernel) and every face (interior penalty + Dirichlet,
    face kernel) into the variable-block matrix.  Then a fixed number of
    GMRES(50) iterations with block Jacobi (the iteration count to 1e-10 grows
    with the mesh; the per-iteration cost is the figure of merit)."""
    from modfem_gb300.mesh import anisotropic_tensors, lognormal_k, prism_faces, structured_prism_mesh
    out = {}
    for name, n, mode in (("p3_anisotropic_432k", 60, "p3"), ("mixed_p1to4_390k", 58, "mixed")):
        m = structured_prism_mesh(n, jitter=0.2, seed=SEED)
        F = prism_faces(m)
        c = gb.Context(local)
        c.set_mesh(m)
        if mode == "p3":
            pdeg = np.full(m.nel, 3)
            c.set_coefficients(D=anisotropic_tensors(m.nel, seed=SEED), f=1.0, g=0.0)
        else:
            pdeg = np.random.default_rng(SEED).integers(1, 5, m.nel)
            c.set_coefficients(k=lognormal_k(m.nel, seed=SEED), f=1.0, g=0.0)
        c.dg_set_degrees(pdeg)
        c.dg_set_faces(F, penalty=10.0)
        nd, nv = c.dg_build_structure()
        tuned_vol, tuned_face, _ = c.dg_autotune(sample=65536)  # launch shapes per degree (results unchanged)
        for _ in range(2):
            c.dg_assemble()
        tt = np.zeros(3)
        for _ in range(steps):
            c.dg_assemble()
            tt += np.array(c.dg_last_timing()[:3])
        tot, vol, fa = tt / steps
        v64, r64 = c.dg_get_matrix()
        # the same assembly with the tensor-core volume kernel (split BF16)
        c.dg_set_volume_kernel(gb.DG_VOLUME_TC)
        c.dg_assemble()
        tt = np.zeros(3)
        for _ in range(steps):
            c.dg_assemble()
            tt += np.array(c.dg_last_timing()[:3])
        tot_tc, vol_tc, _ = tt / steps
        vtc, rtc = c.dg_get_matrix()
        tc_dev = float(np.max(np.abs(vtc - v64)) / np.max(np.abs(v64)))
        del vtc
        # and with the TF32 hi/lo contraction (FP32 accumulation: approximate)
        c.dg_set_volume_kernel(gb.DG_VOLUME_TF32)
        c.dg_assemble()
        tt = np.zeros(3)
        for _ in range(steps):
            c.dg_assemble()
            tt += np.array(c.dg_last_timing()[:3])
        tot_tf, vol_tf, _ = tt / steps
        vtf, _ = c.dg_get_matrix()
        tf_dev = float(np.max(np.abs(vtf - v64)) / np.max(np.abs(v64)))
        del vtf
        # the whole assembly on the tensor cores: split-BF16 volume and faces
        c.dg_set_volume_kernel(gb.DG_VOLUME_TC)
        c.dg_set_face_kernel(gb.DG_FACE_TC)
        c.dg_assemble()
        tt = np.zeros(3)
        for _ in range(steps):
            c.dg_assemble()
            tt += np.array(c.dg_last_timing()[:3])
        tot_ta, vol_ta, fa_ta = tt / steps
        vta, _ = c.dg_get_matrix()
        ta_dev = float(np.max(np.abs(vta - v64)) / np.max(np.abs(v64)))
        del vta
        # double-word sums on the FP32 pipes for volume and faces (all
        # degrees), and the tensor cores where they apply with double words
        # for the rest
        dwf = {}
        for key, vmode, fmode in (("double_word_assembly", gb.DG_VOLUME_DWORD, gb.DG_FACE_DWORD),
                                  ("fastest_assembly", gb.DG_VOLUME_DWORD, gb.DG_FACE_TC_DWORD)):
            c.dg_set_volume_kernel(vmode)
            c.dg_set_face_kernel(fmode)
            c.dg_assemble()
            tt = np.zeros(3)
            for _ in range(steps):
                c.dg_assemble()
                tt += np.array(c.dg_last_timing()[:3])
            tot_tw, vol_tw, fa_tw = tt / steps
            vtw, _ = c.dg_get_matrix()
            dwf[key] = {"volume_ms": vol_tw, "face_ms": fa_tw, "assemble_ms": tot_tw,
                        "elem_per_s": m.nel / (tot_tw * 1e-3), "speedup_vs_fp64": tot / tot_tw,
                        "face_speedup_vs_fp64": fa / fa_tw,
                        "max_abs_diff_vs_fp64_rel_to_max": float(np.max(np.abs(vtw - v64)) / np.max(np.abs(v64)))}
            del vtw
        del v64
        c.dg_set_face_kernel(gb.DG_FACE_FP64)
        c.dg_set_volume_kernel(gb.DG_VOLUME_FP64)
        vfma = sum(dg_fma_per_element(p) * int(np.sum(pdeg == p)) for p in range(1, 5))
        ffma = dg_face_fma(F, pdeg)
        # mixed-precision refinement: the same number of inner iterations on
        # the FP32 operator (per-iteration cost; FP64 outer residual)
        _, it_ir, outer_ir, rel_ir = c.dg_solve_ir(krylov=50, max_iter=gmres_iters, tol_rel=1e-10, inner_tol=1e-4)
        ir_ms = c.last_solve_timing()[0]
        x, it, res, rel = c.dg_solve(krylov=50, max_iter=gmres_iters, tol_rel=1e-10)
        st = c.last_solve_timing()
        spmv_ms = st[1] / max(st[2], 1)
        # the same iterations with the Arnoldi products on double-word copies
        c.set_option(gb.OPT_DG_SPMV_ARITH, gb.STD_DWORD)
        xdw, it_dw, _, rel_dw = c.dg_solve(krylov=50, max_iter=gmres_iters, tol_rel=1e-10)
        st_dw = c.last_solve_timing()
        c.set_option(gb.OPT_DG_SPMV_ARITH, gb.STD_FP64)
        dw_solve = {"gmres_iterations": it_dw, "gmres_ms_per_iteration": st_dw[0] / max(it_dw, 1),
                    "spmv_ms": st_dw[1] / max(st_dw[2], 1), "rel_residual": rel_dw,
                    "solution_rel_diff_vs_fp64": float(np.max(np.abs(xdw - x)) / np.max(np.abs(x)))}
        inv_bytes = 8 * sum(int(np.sum(pdeg == p)) * [0, 6, 18, 40, 75][p] ** 2 for p in range(1, 5))
        out[name] = {
            "elements": m.nel, "faces": int(F.n), "dofs": nd, "stored_values": nv,
            "autotuned_shapes": {"volume": tuned_vol[1:].tolist(), "face": tuned_face[1:].tolist()},
            "assemble_ms": tot, "elem_per_s": m.nel / (tot * 1e-3),
            "volume_ms": vol, "volume_fp64_frac": 2 * vfma / (vol * 1e-3) / 1e12 / fp64_peak,
            "face_ms": fa, "face_fp64_frac": 2 * ffma / (fa * 1e-3) / 1e12 / fp64_peak,
            "tensor_core_volume": {"volume_ms": vol_tc, "assemble_ms": tot_tc, "elem_per_s": m.nel / (tot_tc * 1e-3),
                                   "max_abs_diff_vs_fp64_rel_to_max": tc_dev,
                                   "note": "tcgen05 split-BF16 products (p <= 3; p = 4 stays FP64)"},
            "tensor_core_assembly": {"volume_ms": vol_ta, "face_ms": fa_ta, "assemble_ms": tot_ta,
                                     "elem_per_s": m.nel / (tot_ta * 1e-3), "speedup_vs_fp64": tot / tot_ta,
                                     "max_abs_diff_vs_fp64_rel_to_max": ta_dev,
                                     "note": "tcgen05 split-BF16 volume and faces (owners and neighbours p <= 3; "
                                             "others stay FP64)"},
            "double_word_assembly": dict(
                dwf["double_word_assembly"],
                note="volume and face entries summed in double-word (float pair) arithmetic on the FP32 pipes, "
                     "all degrees"),
            "fastest_assembly": dict(
                dwf["fastest_assembly"],
                note="double-word volume (all degrees); split-BF16 tensor-core faces (owners and neighbours p <= 3), "
                     "double-word faces for the rest"),
            "tf32_volume": {"volume_ms": vol_tf, "assemble_ms": tot_tf, "elem_per_s": m.nel / (tot_tf * 1e-3),
                            "max_abs_diff_vs_fp64_rel_to_max": tf_dev,
                            "note": "tcgen05 kind::tf32, hi/lo operands, FP32 accumulation (p <= 3)"},
            "gmres_iterations": it, "gmres_rel_residual": rel, "gmres_ms_per_iteration": st[0] / max(it, 1),
            "spmv_ms": spmv_ms,
            "gmres_double_word_operator": dw_solve,
            "ir_fp32_inner": {"inner_iterations": it_ir, "refinement_steps": outer_ir,
                              "ms_per_inner_iteration": ir_ms / max(it_ir, 1), "true_rel_residual": rel_ir},
            # the preconditioned block SpMV: matrix + inverted diagonal blocks, one FMA per value
            "spmv_fp64_frac": 2 * (nv + inv_bytes / 8) / (spmv_ms * 1e-3) / 1e12 / fp64_peak,
            "spmv_gbs": (8 * nv + inv_bytes + 24 * nd) / (spmv_ms * 1e-3) / 1e9,
        }
        hbm = hbm_peak_gbs()
        if hbm:
            b = 8 * nv + inv_bytes + 24 * nd
            out[name]["spmv_hbm_frac_of_measured"] = b / (max(spmv_ms, 1e-9) * 1e-3) / 1e9 / hbm
            out[name]["gmres_double_word_operator"]["spmv_hbm_frac_of_measured"] = (
                b / (max(dw_solve["spmv_ms"], 1e-9) * 1e-3) / 1e9 / hbm)
        c.close()
    return out


def tet_fma_per_element(p):
    """FP64 FMAs of the tetrahedron tile per element: 6 per upper entry."""
    ns = (p + 1) * (p + 2) * (p + 3) // 6
    return 6 * ns * (ns + 1) // 2


def bench_batch(gb, local, steps, fp64_peak):
    """Batched mixed elements: 400,000 DG prisms (the first 400k of the
    59^3 x 2 jittered mesh) and 300,000 affine DG tetrahedra (the first 300k
    of the 37^3 x 6 jittered Kuhn mesh), p uniform in 1..4 per element
    (seeded), lognormal(0,1) k.  A step is one replay of the persistent
    mixed-(type, p) volume kernel with autotuned variants per class, writing
    every element block into one variable-block array.  Beside it: the prisms
    through the per-degree kernels (four launches, autotuned shapes) and an
    end-to-end step from host arrays (upload, run, download)."""
    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh, structured_tet_mesh
    NP, NT = 400_000, 300_000
    m = structured_prism_mesh(59, jitter=0.2, seed=SEED)
    t = structured_tet_mesh(37, jitter=0.2, seed=SEED)
    rng = np.random.default_rng(SEED)
    pp = rng.integers(1, 5, NP).astype(np.int32)
    tp = rng.integers(1, 5, NT).astype(np.int32)
    k = lognormal_k(NP + NT, seed=SEED)
    A = k[:, None] * np.eye(3).reshape(1, 9)
    pX = np.ascontiguousarray(m.coords[m.el_nodes[:NP]])
    tX = np.ascontiguousarray(t.coords[t.el_nodes[:NT]])
    b = gb.Batch(local)
    nval, nrhs = b.set(pX, A[:NP], pp, tX, A[NP:], tp, f=1.0)
    pv, tv, tune_ms = b.autotune(sample=32768)
    for _ in range(3):
        b.run()
    ms = [b.run() for _ in range(steps)]
    step_ms = float(np.mean(ms))
    v64, _ = b.get()
    # the same launch with the prism stiffness sums in double-word arithmetic
    b.set_arith(True)
    for _ in range(2):
        b.run()
    dw_ms = float(np.mean([b.run() for _ in range(steps)]))
    vdw, _ = b.get()
    dw_dev = float(np.max(np.abs(vdw - v64)) / np.max(np.abs(v64)))
    del v64, vdw
    b.set_arith(False)
    pfma = sum(dg_fma_per_element(q) * int(np.sum(pp == q)) for q in range(1, 5))
    tfma = sum(tet_fma_per_element(q) * int(np.sum(tp == q)) for q in range(1, 5))
    out_bytes = 8 * (nval + nrhs)
    # the tetrahedra alone (HBM-write bound) and the prisms alone
    bt = gb.Batch(local)
    bt.set(np.zeros((0, 6, 3)), np.zeros((0, 9)), np.zeros(0, np.int32), tX, A[NP:], tp, f=1.0)
    bt.set_variants(None, tv)
    bt.run()
    tet_ms = float(np.mean([bt.run() for _ in range(steps)]))
    tnv, tnr = bt.nval, bt.nrhs
    bt.close()
    # end to end from host arrays: set (upload + tile build), run, download
    hv, hr = gb.PinnedArray((nval,)), gb.PinnedArray((nrhs,))
    hin = []
    for arr in (pX, A[:NP], pp, tX, A[NP:], tp):
        h = gb.PinnedArray(arr.shape, arr.dtype)
        h.array[...] = arr
        hin.append(h)
    e2e = []
    for _ in range(2):
        t0 = time.perf_counter()
        b.set(*[h.array for h in hin], f=1.0)
        b.set_variants(pv, tv)
        b.run()
        b.L.gbfem_batch_get(b._h, hv.array.ctypes.data, hr.array.ctypes.data)
        e2e.append(time.perf_counter() - t0)
    e2e_s = min(e2e)
    for h in hin + [hv, hr]:
        h.free()
    b.close()
    # prisms through the per-degree kernels (volume only, no faces)
    class _M:
        pass
    pm = _M()
    pm.coords, pm.el_nodes = m.coords, np.ascontiguousarray(m.el_nodes[:NP])
    pm.bc_face_id = pm.bc_face_el = pm.bc_face_side = pm.bc_face_bc = np.zeros(0, np.int32)
    c = gb.Context(local)
    c.set_mesh(pm)
    c.set_coefficients(k=k[:NP], f=1.0, g=0.0)
    c.dg_set_degrees(pp)
    c.dg_build_structure()
    c.dg_autotune(sample=65536)
    c.dg_assemble()
    vol = []
    for _ in range(steps):
        c.dg_assemble()
        vol.append(c.dg_last_timing()[1])
    per_degree_ms = float(np.mean(vol))
    c.close()
    return {
        "workload": f"{NP} DG prisms + {NT} affine DG tetrahedra, p uniform 1..4, lognormal k, one persistent launch",
        "elements": NP + NT, "stored_values": nval, "rhs": nrhs,
        "autotuned_variants": {"prism": pv[1:].tolist(), "tet_elements_per_tile": [8 << int(v) for v in tv[1:]]},
        "step_ms": step_ms, "elem_per_s": (NP + NT) / (step_ms * 1e-3),
        "fp64_frac": 2 * (pfma + tfma) / (step_ms * 1e-3) / 1e12 / fp64_peak,
        "output_gbs": out_bytes / (step_ms * 1e-3) / 1e9,
        "tets_alone_ms": tet_ms, "tets_alone_output_gbs": 8 * (tnv + tnr) / (tet_ms * 1e-3) / 1e9,
        "prisms_per_degree_kernels_ms": per_degree_ms,
        "double_word_prisms": {"step_ms": dw_ms, "elem_per_s": (NP + NT) / (dw_ms * 1e-3),
                               "speedup_vs_fp64": step_ms / dw_ms, "max_abs_diff_vs_fp64_rel_to_max": dw_dev,
                               "note": "prism stiffness sums in double-word (float pair) arithmetic, tetrahedra FP64"},
        "e2e_ms": e2e_s * 1e3, "e2e_elem_per_s": (NP + NT) / e2e_s,
        "e2e_note": "page-locked host arrays: upload of geometry and tensors, tile build, graph capture, run, "
                    "download of "
                    f"{out_bytes / 1e9:.2f} GB of blocks",
    }


def bench_tet_dg(gb, local, steps):
    """The tetrahedral part of the mixed prism + tetrahedron workload as a
    DG system: 37^3 x 6 = 303,918
    jittered affine tetrahedra, p uniform in 1..4 (seeded), lognormal(0,1)
    k, interior-penalty faces (616,050 faces) into the variable-block
    storage; then a fixed 100 GMRES(50) iterations with block Jacobi."""
    from modfem_gb300.mesh import lognormal_k, structured_tet_mesh, tet_faces
    t = structured_tet_mesh(37, jitter=0.2, seed=SEED)
    F = tet_faces(t)
    p = np.random.default_rng(SEED).integers(1, 5, t.nel)
    c = gb.Context(local)
    c.set_mesh(t)
    c.set_coefficients(k=lognormal_k(t.nel, seed=SEED), f=1.0, g=0.0)
    c.dg_set_degrees(p)
    c.dg_set_faces(F, penalty=10.0)
    nd, nv = c.dg_build_structure()
    for _ in range(2):
        c.dg_assemble()
    tt = np.zeros(3)
    for _ in range(steps):
        c.dg_assemble()
        tt += np.array(c.dg_last_timing()[:3])
    tot, vol, fa = tt / steps
    v64, _ = c.dg_get_matrix()
    # the faces summed in double-word arithmetic
    c.dg_set_face_kernel(gb.DG_FACE_DWORD)
    c.dg_assemble()
    tt = np.zeros(3)
    for _ in range(steps):
        c.dg_assemble()
        tt += np.array(c.dg_last_timing()[:3])
    tot_dw, _, fa_dw = tt / steps
    vdw, _ = c.dg_get_matrix()
    dw_dev = float(np.max(np.abs(vdw - v64)) / np.max(np.abs(v64)))
    del v64, vdw
    c.dg_set_face_kernel(gb.DG_FACE_FP64)
    c.dg_assemble()
    x, it, res, rel = c.dg_solve(krylov=50, max_iter=100, tol_rel=1e-10)
    st = c.last_solve_timing()
    out = {"elements": t.nel, "faces": int(F.n), "dofs": nd, "stored_values": nv,
           "assemble_ms": tot, "volume_ms": vol, "face_ms": fa, "elem_per_s": t.nel / (tot * 1e-3),
           "double_word_faces": {"face_ms": fa_dw, "assemble_ms": tot_dw, "face_speedup_vs_fp64": fa / fa_dw,
                                 "max_abs_diff_vs_fp64_rel_to_max": dw_dev},
           "gmres_iterations": it, "gmres_ms_per_iteration": st[0] / max(it, 1),
           "spmv_ms": st[1] / max(st[2], 1)}
    c.close()
    return out


def bench_mixed_dg_system(gb, local, steps, n=63, layers=50):
    """Config 3 as one DG system on one connected mesh: 63^3 hexahedra, the
    lower 50 layers split into 2 prisms each (396,900 jittered prisms), the
    upper 13 into 6 tetrahedra each (309,582 affine tetrahedra), the two
    regions joined by 7,938 prism-tetrahedron triangles; p uniform in 1..4
    (seeded), lognormal(0,1) k, interior-penalty faces into the
    variable-block storage.  Assembly (volume and all faces) in plain FP64
    and in the fastest form (double-word volume sums, split-BF16 tensor-core
    faces between prisms), then a fixed 100 GMRES(50) iterations with block
    Jacobi."""
    from modfem_gb300.mesh import lognormal_k, mixed_faces, structured_mixed_mesh
    m = structured_mixed_mesh(n, layers, jitter=0.2, seed=SEED)
    F = mixed_faces(m)
    p = np.random.default_rng(SEED).integers(1, 5, m.nel)
    c = gb.Context(local)
    c.set_mesh_mixed(m)
    c.set_coefficients(k=lognormal_k(m.nel, seed=SEED), f=1.0, g=0.0)
    c.dg_set_degrees(p)
    c.dg_set_faces(F, penalty=10.0)
    nd, nv = c.dg_build_structure()
    out = {"prisms": int((m.el_nv == 6).sum()), "tetrahedra": int((m.el_nv == 4).sum()), "faces": int(F.n),
           "prism_tetrahedron_faces": int(((F.el2 >= 0) & (m.el_nv[F.el1] != m.el_nv[np.maximum(F.el2, 0)])).sum()),
           "dofs": nd, "stored_values": nv}
    v64 = None
    for key, vol, face in (("fp64", gb.DG_VOLUME_FP64, gb.DG_FACE_FP64),
                           ("fastest", gb.DG_VOLUME_DWORD, gb.DG_FACE_TC_DWORD)):
        c.dg_set_volume_kernel(vol)
        c.dg_set_face_kernel(face)
        for _ in range(2):
            c.dg_assemble()
        tt = np.zeros(3)
        launches = 0
        for _ in range(steps):
            c.dg_assemble()
            t = c.dg_last_timing()
            tt += np.array(t[:3])
            launches = t[3]
        tot, vol_ms, fa = tt / steps
        r = {"assemble_ms": tot, "volume_ms": vol_ms, "face_ms": fa, "elem_per_s": m.nel / (tot * 1e-3),
             "launches": launches}
        vals, _ = c.dg_get_matrix()
        if v64 is None:
            v64 = vals
        else:
            r["max_abs_diff_vs_fp64_rel_to_max"] = float(np.max(np.abs(vals - v64)) / np.max(np.abs(v64)))
            r["speedup_vs_fp64"] = out["fp64"]["assemble_ms"] / tot
        del vals
        out[key] = r
    del v64
    c.dg_set_volume_kernel(gb.DG_VOLUME_FP64)
    c.dg_set_face_kernel(gb.DG_FACE_FP64)
    c.dg_assemble()
    x, it, res, rel = c.dg_solve(krylov=50, max_iter=100, tol_rel=1e-10)
    st = c.last_solve_timing()
    out.update({"elements": m.nel, "gmres_iterations": it, "gmres_ms_per_iteration": st[0] / max(it, 1),
                "spmv_ms": st[1] / max(st[2], 1)})
    c.close()
    return out


def mixed_precision_solution_check(gb, local, sizes=(10, 16)):
    """Config-4 form at sizes GMRES(50) converges on in a bench run: p = 3
    prisms, the anisotropic tensor, Dirichlet value 0.3.  Every assembly
    (plain FP64; split-BF16 tensor-core volume and faces; double-word volume
    with tensor-core faces; double-word volume and faces) is solved by FP64
    iterative refinement around FP32-operator GMRES(50) with compensated
    residuals until the corrections reach FP64 rounding, so each solution is
    its matrix's to ~1e-15 and the differences are the matrices' effect on
    the solution.  Reported: relative solution error (2-norm) of each mixed
    form against the plain FP64 assembly's solution, and the plain FP64
    GMRES (stopped at 1e-12 preconditioned) against the same."""
    from modfem_gb300.mesh import anisotropic_tensors, prism_faces, structured_prism_mesh
    forms = {"fp64": (gb.DG_VOLUME_FP64, gb.DG_FACE_FP64), "tc_volume_tc_faces": (gb.DG_VOLUME_TC, gb.DG_FACE_TC),
             "dword_volume_tc_faces": (gb.DG_VOLUME_DWORD, gb.DG_FACE_TC),
             "dword_volume_dword_faces": (gb.DG_VOLUME_DWORD, gb.DG_FACE_DWORD)}
    out, summary = {}, {}
    for n in sizes:
        m = structured_prism_mesh(n, jitter=0.2, seed=44)
        F = prism_faces(m)
        D = anisotropic_tensors(m.nel, seed=44)
        res, xs = {"elements": m.nel}, {}
        for name, (vol, face) in forms.items():
            c = gb.Context(local)
            c.set_mesh(m)
            c.set_coefficients(D=D, f=1.0, g=0.3)
            c.dg_set_degrees(np.full(m.nel, 3))
            c.dg_set_faces(F, penalty=10.0)
            c.dg_build_structure()
            c.dg_set_volume_kernel(vol)
            c.dg_set_face_kernel(face)
            c.dg_assemble()
            c.set_option(gb.OPT_DG_RESIDUAL, gb.RESIDUAL_COMPENSATED)
            x, it, outer, rel = c.dg_solve_ir(krylov=50, max_iter=400000, tol_rel=1e-300, inner_tol=1e-6)
            res[name] = {"inner_iterations": it, "refinements": outer, "true_rel_residual": rel,
                         "solve_ms": c.last_solve_timing()[0]}
            xs[name] = np.array(x)
            if name == "fp64":
                xg, itg, _, relg = c.dg_solve(krylov=50, max_iter=400000, tol_rel=1e-12)
                res["fp64_gmres_1e-12"] = {"iterations": itg, "solve_ms": c.last_solve_timing()[0],
                                           "rel_solution_error_vs_refined": float(np.linalg.norm(xg - x) /
                                                                                  np.linalg.norm(x))}
            c.close()
        for name in forms:
            if name != "fp64":
                res[name]["rel_solution_error_vs_fp64"] = float(np.linalg.norm(xs[name] - xs["fp64"]) /
                                                                np.linalg.norm(xs["fp64"]))
        out[f"n{n}"] = res
        summary[f"{m.nel}_prisms"] = {name: _r(res[name]["rel_solution_error_vs_fp64"], 3) for name in forms
                                      if name != "fp64"}
        summary[f"{m.nel}_prisms"]["fp64_gmres_1e-12"] = _r(res["fp64_gmres_1e-12"]["rel_solution_error_vs_refined"], 3)
    out["summary"] = {"rel_solution_error_vs_fp64": summary, "bound": 1e-10,
                      "note": "each assembly solved by compensated-residual refinement to FP64 rounding"}
    return out


def bench_serving(gb, local, rates=(50, 200, 1000, 2000), per_rate=48):
    """The serving workload: a Poisson stream of independent heat problems,
    each a structured prism mesh of n^3 hexahedra x 2 with n log-uniform in
    [10, 60] (a stratified sample of 8 sizes), lognormal(0,1) k, f = 1,
    solved by GMRES(30) to 1e-8.  Half the requests are std linear; the
    other half DG with p in {1, 2}, whose n is drawn from [10, 20] (GMRES(30)
    with block Jacobi needs more than 3,000 iterations, seconds per request,
    beyond that).  Beside the engine: the
    plain one-at-a-time path (gbfem Context per request: upload, structure,
    assemble, solve) with its measured service times queued FIFO on the same
    arrival times."""
    from modfem_gb300.mesh import lognormal_k, prism_faces, structured_prism_mesh
    from modfem_gb300.serve import DG, STD, Problem, Server, poisson_stream
    # 16 problems, alternating std and DG; n stratified over the log-uniform
    # distribution (the i-th of 8 at quantile (i + 1/2) / 8, in a seeded
    # order), so the pool holds its share of >= 100k-element std requests
    rng = np.random.default_rng(SEED)
    qs = rng.permutation(8)
    pool = []
    for i in range(16):
        kind = STD if i % 2 == 0 else DG
        hi = 60 if kind == STD else 20
        n = int(round(10.0 * (hi / 10.0) ** ((qs[i // 2] + 0.5) / 8)))
        p = 1 if i % 4 == 1 else 2
        m = structured_prism_mesh(n, jitter=0.2, seed=1000 + i)
        k = lognormal_k(m.nel, seed=2000 + i)
        F = prism_faces(m) if kind == DG else None
        pool.append((m, k, F, Problem(m, k, kind=kind, p=p, faces=F, krylov=30, max_iter=20000, tol=1e-8)))
    # plain one-at-a-time service times
    service = []
    for (m, k, F, pr) in pool:
        t0 = time.perf_counter()
        c = gb.Context(local)
        c.set_mesh(m)
        c.set_coefficients(k=k, f=1.0, g=0.0)
        if pr.kind == DG:
            c.dg_set_degrees(np.full(m.nel, pr.p))
            c.dg_set_faces(F, penalty=10.0)
            c.dg_build_structure()
            c.dg_assemble()
            c.dg_solve(krylov=30, max_iter=20000, tol_rel=1e-8)
        else:
            c.build_structure()
            c.assemble()
            c.solve(krylov=30, max_iter=20000, tol_rel=1e-8)
        c.close()
        service.append(time.perf_counter() - t0)
    srv = Server(local, max_active=32, prep_threads=8)
    out = {"requests_per_rate": per_rate, "pool": [{"kind": "std" if pr.kind == STD else f"dg_p{pr.p}",
                                                     "elements": int(m.nel)} for (m, _, _, pr) in pool],
           "rates": []}
    try:
        poisson_stream(srv, [pr for (_, _, _, pr) in pool], 1000.0, 12, seed=1)  # warm-up
        for rate in rates:
            res, span = poisson_stream(srv, [pr for (_, _, _, pr) in pool], rate, per_rate, seed=rate)
            lat = np.array([r["latency"] for r in res])
            big = np.array([r["latency"] for r in res if r["nel"] >= 80000 and r["kind"] == STD])
            b100 = [r for r in res if r["nel"] >= 100000 and r["kind"] == STD]
            l100 = np.array([r["latency"] for r in b100])
            # where the large std requests' time goes: admission queue,
            # preparation, wait for the engine, GMRES (means over them)
            parts = (np.mean([r["times"][:4] for r in b100], axis=0) * 1e3).tolist() if b100 else None
            # the plain path on the same arrivals
            arr = np.cumsum(np.random.default_rng(rate).exponential(1.0 / rate, per_rate))
            fin, plain = 0.0, []
            for i in range(per_rate):
                fin = max(arr[i], fin) + service[i % len(pool)]
                plain.append(fin - arr[i])
            plain = np.array(plain)
            out["rates"].append({
                "rate_req_s": rate, "p50_ms": 1e3 * float(np.percentile(lat, 50)),
                "p99_ms": 1e3 * float(np.percentile(lat, 99)), "problems_per_s": per_rate / span,
                "p99_ms_std_over_80k_elements": 1e3 * float(np.percentile(big, 99)) if big.size else None,
                "p99_ms_std_100k": 1e3 * float(np.percentile(l100, 99)) if l100.size else None,
                "p50_ms_std_100k": 1e3 * float(np.percentile(l100, 50)) if l100.size else None,
                "std_100k_requests": int(l100.size),
                "std_100k_mean_ms_queue_prep_wait_solve": parts,
                "plain_one_at_a_time": {"p50_ms": 1e3 * float(np.percentile(plain, 50)),
                                        "p99_ms": 1e3 * float(np.percentile(plain, 99)),
                                        "problems_per_s": per_rate / (max(fin, arr[-1]))}})
        out["engine"] = srv.stats()
    finally:
        srv.close()
    return out


def run_reference(args, ws, rank):
    if rank != 0:
        return
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "liboracle.so"])
    m, k = make_problem(args.n)
    nthreads = os.cpu_count() or 1
    cpu_assemble(m, k, nthreads, reps=args.warmup)
    times, _, _ = cpu_assemble(m, k, nthreads, reps=args.steps)
    t = sum(times) / len(times)
    v = m.nel / t
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded mesh jitter and k)",
        "config": {"workload": f"std P1 prism integrate+assemble, {args.n}^3 hex x 2 = {m.nel} prisms, "
                               f"lognormal(0,1) k, +-0.2h jitter, penalty Dirichlet",
                   "parallelism": "CPU host threads"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": f"full {m.nel}-element assembly per step (colour-parallel OpenMP)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _r(x, d=4):
    """Rounds to d significant digits (None passes)."""
    if x is None or not isinstance(x, (int, float)):
        return x
    return float(f"{x:.{d}g}")


def compact_line(full):
    """The contract keys plus the summaries the headline rests on, a few KB:
    the plain FP64 path, precision, the std solver, the DG p = 3 and mixed
    assemblies, the mixed-precision solution error, the batch and serving
    summaries.  The whole record goes to the detail file (BENCH_DETAIL, by
    default bench_detail.json beside this script)."""
    keep = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
            "vs_baseline", "dtype", "data", "config", "roofline", "cpu_baseline", "e2e", "clocks", "gpu_launches",
            "speedup_vs_plain_fp64")
    out = {k: full[k] for k in keep if k in full}
    pf = full["plain_fp64"]
    out["plain_fp64"] = {"value": pf["value"], "e2e": pf["e2e"]["value"], "element_kernel_ms": pf["element_kernel_ms"],
                         "roofline_frac_fp64": _r(pf["roofline"]["frac"]),
                         "fp64_pipe_slot_frac": _r(pf["roofline"]["fp64_pipe_slot_frac"]),
                         "fp64_peak_tflops_measured": _r(pf["roofline"]["peak"])}
    pr = full["precision"]
    out["precision"] = {"bound_rel": pr["bound_rel"],
                        "dword_vs_fp64_energy": _r(pr["max_rel_err_vs_plain_fp64_energy_scale"], 3),
                        "vs_oracle_energy": {k: _r(v, 3) for k, v in
                                             pr.get("max_rel_err_vs_oracle_energy_scale", {}).items()}}
    sv = full["solver"]
    skeys = ("spmv_ms", "spmv_gbs", "spmv_hbm_frac_of_measured", "gmres_ms_per_iteration", "gmres_iterations",
             "gmres_to_1e-8_ms", "gmres_to_1e-8_iterations")
    out["solver"] = {k: _r(sv.get(k)) for k in skeys}
    if "double_word_spmv" in sv:
        out["solver"]["double_word_spmv"] = {k: _r(sv["double_word_spmv"].get(k)) for k in skeys}
    if "e2e_cold" in full:
        out["e2e_cold"] = full["e2e_cold"]
    dg = full["dg"]
    for key, name in (("dg_p3_432k", "p3_anisotropic_432k"), ("dg_mixed_p1to4_390k", "mixed_p1to4_390k")):
        d = dg.get(name)
        if not d:
            continue
        out[key] = {"fp64_assemble_ms": _r(d["assemble_ms"]), "fp64_volume_frac": _r(d["volume_fp64_frac"], 3),
                    "fp64_face_frac": _r(d["face_fp64_frac"], 3)}
        for form in ("tensor_core_assembly", "double_word_assembly", "fastest_assembly"):
            f = d[form]
            out[key][form] = {"assemble_ms": _r(f["assemble_ms"]), "face_ms": _r(f["face_ms"]),
                              "speedup_vs_fp64": _r(f["speedup_vs_fp64"], 3),
                              "max_dev_rel_to_max": _r(f["max_abs_diff_vs_fp64_rel_to_max"], 2)}
        out[key]["spmv_hbm_frac_of_measured"] = _r(d.get("spmv_hbm_frac_of_measured"), 3)
        out[key]["gmres_ms_per_iteration"] = _r(d["gmres_ms_per_iteration"])
    mps = dg.get("mixed_precision_solution")
    if mps:
        out["mixed_precision_solution"] = mps.get("summary", mps)
    b = full["batch_mixed"]
    out["batch_mixed"] = {"step_ms": _r(b["step_ms"]), "elem_per_s": _r(b["elem_per_s"]),
                          "fp64_frac": _r(b["fp64_frac"], 3),
                          "double_word_step_ms": _r(b["double_word_prisms"]["step_ms"])}
    # the mixed prism + tetrahedron workload as a whole step: the mixed-degree prism DG system and
    # the tetrahedral DG system (volume and faces each, measured above in this
    # run; the two element types form separate systems, no prism-tetrahedron
    # faces)
    mx, tet = dg.get("mixed_p1to4_390k"), b.get("tet_dg_system")
    if mx and tet:
        out["batch_mixed"]["config3_whole_step_ms"] = {
            "fp64": _r(mx["assemble_ms"] + tet["assemble_ms"]),
            "double_word": _r(mx["double_word_assembly"]["assemble_ms"] + tet["double_word_faces"]["assemble_ms"]),
            "elements": mx["elements"] + tet["elements"]}
    # the same workload as one system on one connected prism + tetrahedron mesh
    ms = b.get("mixed_dg_system")
    if ms:
        out["batch_mixed"]["config3_one_system"] = {
            "elements": ms["elements"], "prism_tetrahedron_faces": ms["prism_tetrahedron_faces"],
            "fp64_assemble_ms": _r(ms["fp64"]["assemble_ms"]), "fastest_assemble_ms": _r(ms["fastest"]["assemble_ms"]),
            "fastest_max_dev_rel_to_max": _r(ms["fastest"]["max_abs_diff_vs_fp64_rel_to_max"], 2),
            "gmres_ms_per_iteration": _r(ms["gmres_ms_per_iteration"])}
    sv = full.get("serving")
    if sv:
        out["serving"] = {"p50_ms": {str(r["rate_req_s"]): _r(r["p50_ms"]) for r in sv["rates"]},
                          "p50_ms_std_100k": {str(r["rate_req_s"]): _r(r.get("p50_ms_std_100k")) for r in sv["rates"]},
                          "p99_ms": {str(r["rate_req_s"]): _r(r["p99_ms"]) for r in sv["rates"]},
                          "p99_ms_std_100k": {str(r["rate_req_s"]): _r(r.get("p99_ms_std_100k")) for r in sv["rates"]},
                          "problems_per_s": {str(r["rate_req_s"]): _r(r["problems_per_s"]) for r in sv["rates"]},
                          "plain_p99_ms": {str(r["rate_req_s"]): _r(r["plain_one_at_a_time"]["p99_ms"])
                                           for r in sv["rates"]}}
    out["detail_file"] = os.path.relpath(DETAIL_FILE, ROOT)
    return out


def main():
    args = parse()
    if args.profile:
        from modfem_gb300 import build
        build.build(verbose=False)
        args.n = args.n if args.n != N_HEX else 24
        run_profile_case(args)
        return
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    import modfem_gb300 as gb
    from modfem_gb300 import build
    if rank == 0:
        build.build(verbose=False)
    barrier(ws)

    m, k = make_problem(args.n)
    c = gb.Context(local)
    c.set_mesh(m)
    c.set_coefficients(k=k, f=1.0, g=0.0, penalty=1e7)
    # structure (setup, not in the timed step): device build, then the host
    # build (which also colours the elements for the deterministic scatter)
    t0 = time.perf_counter()
    c.build_structure_device()
    structure = {"device_build_ms": 1e3 * (time.perf_counter() - t0)}
    t0 = time.perf_counter()
    nd, nnz, ncol = c.build_structure()
    structure["host_build_ms_with_colouring"] = 1e3 * (time.perf_counter() - t0)
    fp64_peak = c.measure_fp64_peak()

    # ---------------- device-resident throughput ----------------
    # the plain FP64 element kernel (the drop-in default), then the
    # double-word one (float pairs, the headline): same mesh, same scatter
    def device_loop(arith):
        c.set_option(gb.OPT_STD_ARITH, arith)
        for _ in range(args.warmup):
            c.assemble(gb.SCATTER_ATOMIC)
        barrier(ws)
        tot, el, nl_sum = 0.0, 0.0, 0
        t0 = time.perf_counter()
        for _ in range(args.steps):
            c.assemble(gb.SCATTER_ATOMIC)
            a, b, nl = c.last_timing()
            tot += a
            el += b
            nl_sum += nl
        wall_ = time.perf_counter() - t0
        return (max_over_ranks(tot / args.steps, ws), max_over_ranks(el / args.steps, ws), nl_sum, wall_,
                c.get_matrix())

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.25)  # let the sampler's first reading land inside the timed region
    ms64, el64, launches64, _, (v64, r64) = device_loop(gb.STD_FP64)
    ms_step, el_ms_step, launches, wall, (vdw, rdw) = device_loop(gb.STD_DWORD)
    value = ws * m.nel / (ms_step * 1e-3)
    value64 = ws * m.nel / (ms64 * 1e-3)
    dn_, rp_, ci_ = c.get_crs_structure()
    rows_ = np.repeat(np.arange(nd), np.diff(rp_))
    isd_ = rows_ == ci_

    def energy_err(a, b):
        diag = np.zeros(nd)
        diag[rows_[isd_]] = np.abs(b[isd_])
        es = np.sqrt(diag[rows_] * diag[ci_])
        return float(np.max(np.abs(a - b) / np.where(es > 0, es, 1.0)))

    precision = {
        "element_arithmetic": "double-word float pairs (about 48 significant bits); FP64 vertex differences, "
                              "FP64 atomic assembly sums",
        "bound_rel": 1e-10,
        "max_rel_err_vs_plain_fp64_energy_scale": energy_err(vdw, v64),
        "max_abs_err_vs_plain_fp64_over_max_entry": float(np.max(np.abs(vdw - v64)) / np.max(np.abs(v64))),
        "rhs_max_rel_err_vs_plain_fp64": float(np.max(np.abs(rdw - r64)) / np.max(np.abs(r64)))}
    assert precision["max_rel_err_vs_plain_fp64_energy_scale"] <= 1e-10

    # ---------------- end to end through the drop-in C ABI ----------------
    tables = c.get_element_tables()
    fa_tab = tables.reshape(m.nel, 42)[m.bc_face_el].reshape(-1)
    ids = np.concatenate([np.arange(1, m.nel + 1), m.bc_face_id]).astype(np.int32)
    types = np.concatenate([np.full(m.nel, gb.ELEMENT), np.full(m.bc_face_id.size, gb.FACE)]).astype(np.int32)
    pos = (np.arange(ids.size) * 42).astype(np.int32)
    table = np.concatenate([tables, fa_tab]).astype(np.int32)
    ce = np.array([0, m.nel], np.int32)
    cf = np.array([m.nel, ids.size], np.int32)
    pins = {}
    for name, arr in (("types", types), ("ids", ids), ("pos", pos), ("table", table), ("ce", ce), ("cf", cf),
                      ("xyz", m.coords), ("k", k)):
        pa = gb.PinnedArray(arr.shape, arr.dtype)
        pa.array[...] = arr
        pins[name] = pa
    out_val = gb.PinnedArray((nnz,))
    out_rhs = gb.PinnedArray((nd,))
    c.set_option(gb.OPT_CACHE_TABLES, 1)
    c.set_option(gb.OPT_STD_ARITH, gb.STD_DWORD)

    def e2e_step():
        c.set_node_coords(pins["xyz"].array)
        c.set_coefficients(k=pins["k"].array, f=1.0, g=0.0, penalty=1e7)
        c.create_assemble_stiff_mat(pins["types"].array, pins["ids"].array, pins["ce"].array, pins["cf"].array,
                                    pins["pos"].array, pins["table"].array, crs_val=out_val.array,
                                    rhs=out_rhs.array)

    for _ in range(max(args.warmup, 1)):
        e2e_step()
    barrier(ws)
    et = []
    for _ in range(args.steps):
        t1 = time.perf_counter()
        e2e_step()
        et.append(time.perf_counter() - t1)
    e2e_s = max_over_ranks(sum(et) / len(et), ws)
    e2e_value = ws * m.nel / e2e_s
    h2d = m.coords.nbytes + k.nbytes
    d2h = 8 * nnz + 8 * nd
    # parity of the e2e result against the device-resident one (same kernels)
    assert np.max(np.abs(out_val.array - vdw)) <= 1e-12 * np.max(np.abs(vdw))
    # cold calls: the cache voided before every step, so the entity lists and
    # the assembly table cross the host link inside the timed call too
    etc = []
    for _ in range(min(args.steps, 10)):
        c.invalidate_tables()
        t1 = time.perf_counter()
        e2e_step()
        etc.append(time.perf_counter() - t1)
    e2e_cold_s = max_over_ranks(sum(etc) / len(etc), ws)
    table_bytes = types.nbytes + ids.nbytes + pos.nbytes + table.nbytes
    assert np.max(np.abs(out_val.array - vdw)) <= 1e-12 * np.max(np.abs(vdw))
    # the same through the plain FP64 kernel
    c.set_option(gb.OPT_STD_ARITH, gb.STD_FP64)
    for _ in range(max(args.warmup, 1)):
        e2e_step()
    et64 = []
    for _ in range(args.steps):
        t1 = time.perf_counter()
        e2e_step()
        et64.append(time.perf_counter() - t1)
    e2e64_s = max_over_ranks(sum(et64) / len(et64), ws)
    assert np.max(np.abs(out_val.array - v64)) <= 1e-12 * np.max(np.abs(v64))
    clocks = sampler.stop()

    # ---------------- GMRES(30) + Jacobi on the assembled matrix ----------------
    # device-resident GMRES (CUDA-graph restart cycles, sliced-ELL SpMV):
    # a fixed 300 iterations for the per-iteration cost, then a solve to
    # 1e-8; with the SpMV in FP64 and in double words
    c.assemble(gb.SCATTER_ATOMIC)
    spmv_bytes = 12 * nnz + 16 * nd
    solver = {"spmv_bytes": spmv_bytes,
              "note": "GMRES(30) + point Jacobi, device-resident (restart cycles replayed as CUDA graphs); "
                      "SpMV on a SELL-32 copy of the CRS matrix"}
    for arith, key in ((gb.STD_FP64, "fp64"), (gb.STD_DWORD, "double_word")):
        c.set_option(gb.OPT_STD_SPMV_ARITH, arith)
        _, it, res, rel = c.solve(30, 300, 1e-14)
        solve_ms, spmv_ms, nspmv, solve_kernels = c.last_solve_timing()
        r = {"gmres_iterations": it, "gmres_ms_per_iteration": solve_ms / max(it, 1),
             "spmv_ms": spmv_ms / max(nspmv, 1), "spmv_gbs": spmv_bytes * nspmv / (spmv_ms * 1e-3) / 1e9,
             "relative_residual_after": rel, "kernel_launches": solve_kernels}
        if hbm_peak_gbs():
            r["spmv_hbm_frac_of_measured"] = r["spmv_gbs"] / hbm_peak_gbs()
        _, it8, _, rel8 = c.solve(30, 20000, 1e-8)
        r["gmres_to_1e-8_iterations"] = it8
        r["gmres_to_1e-8_ms"] = c.last_solve_timing()[0]
        r["gmres_to_1e-8_rel_residual"] = rel8
        if key == "fp64":
            solver.update(r)
        else:
            solver["double_word_spmv"] = r
    c.set_option(gb.OPT_STD_SPMV_ARITH, gb.STD_FP64)

    # ---------------- DG prism system ----------------
    dg = bench_dg(gb, local, max(3, min(args.steps, 10)), fp64_peak)
    batch = bench_batch(gb, local, max(3, min(args.steps, 10)), fp64_peak)
    dg["mixed_precision_solution"] = mixed_precision_solution_check(gb, local)
    batch["tet_dg_system"] = bench_tet_dg(gb, local, max(3, min(args.steps, 10)))
    batch["mixed_dg_system"] = bench_mixed_dg_system(gb, local, max(3, min(args.steps, 10)))

    # ---------------- serving ----------------
    serving = bench_serving(gb, local) if rank == 0 else None

    # ---------------- CPU baseline (rank 0, N=1 only) ----------------
    cpu = None
    if rank == 0 and ws == 1:
        subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "liboracle.so"])
        nthreads = os.cpu_count() or 1
        # the reference arm's procedure on a shorter sample: warm-up runs
        # (thread pool, first-touch of the output arrays), then the mean of
        # the timed ones
        cpu_assemble(m, k, nthreads, reps=2)
        times, vo, ro = cpu_assemble(m, k, nthreads, reps=5)
        tc = sum(times) / len(times)
        precision["max_rel_err_vs_oracle_energy_scale"] = {"double_word": energy_err(vdw, vo),
                                                           "plain_fp64": energy_err(v64, vo)}
        precision["rhs_max_rel_err_vs_oracle"] = {
            "double_word": float(np.max(np.abs(rdw - ro)) / np.max(np.abs(ro))),
            "plain_fp64": float(np.max(np.abs(r64 - ro)) / np.max(np.abs(ro)))}
        del vo, ro
        cpu = {"value": m.nel / tc, "unit": UNIT, "cores": nthreads, "kind": "port",
               "sample": f"mean of 5 full {m.nel}-element integrate+assemble runs (elements + faces) after 2 "
                         "warm-up runs, colour-parallel OpenMP"}

    # plain FP64 kernel: FP64-pipe roofline
    traffic = read_profile_traffic()
    achieved64 = FLOP_PER_ELEM * m.nel / (el64 * 1e-3) / 1e12
    slot_frac = 2 * FP64_SLOTS_PER_ELEM * m.nel / (el64 * 1e-3) / 1e12 / fp64_peak
    # double-word kernel: instruction-issue roofline (4 warp instructions per
    # clock per SM), its instruction count per element from the ncu capture
    dw_prof = read_profile_values("std_prism_elements_dw_686k.md")
    inst_per_elem = dw_prof.get("thread_instructions_per_element")
    digest = source_digest(STD_KERNEL_SOURCES)
    profile_current = dw_prof.get("source_sha256") == digest
    nsm = sm_count(local)
    sm_mhz = (clocks or {}).get("sm_mhz") or 2070.0
    issue_peak = nsm * 4 * 32 * sm_mhz * 1e6 / 1e12
    achieved_issue = inst_per_elem * m.nel / (el_ms_step * 1e-3) / 1e12 if inst_per_elem else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32x2+f64",
        "data": "synthetic (seeded mesh jitter and lognormal k)",
        "config": {"workload": f"std P1 prism integrate+assemble, {args.n}^3 hex x 2 = {m.nel} prisms "
                               f"({nd} dofs, nnz {nnz}, {m.bc_face_id.size} penalty faces), lognormal(0,1) k, "
                               f"+-0.2h jitter",
                   "element_arithmetic": "double-word (float pairs) element matrices, FP64 vertex differences",
                   "scatter": "FP64 atomics", "l2": "inputs larger than L2 (tables 336 MB, values 170 MB)",
                   "parallelism": f"replicas x{ws}" if ws > 1 else "1 GPU"},
        "roofline": {"bound": "issue", "achieved": achieved_issue, "peak": issue_peak, "unit": "Tinst/s",
                     "frac": achieved_issue / issue_peak if achieved_issue else None,
                     "traffic": dw_prof.get("dram_bytes_per_launch"),
                     "kernel": "prism_elements_dw_kernel", "kernel_ms": el_ms_step,
                     "inst_per_elem": inst_per_elem,
                     "inst_source": ("ncu summary profiles/std_prism_elements_dw_686k.md, source digest "
                                     f"{digest} {'matches' if profile_current else 'DIFFERS: stale'}"),
                     "hbm_frac": (ALG_BYTES_PER_ELEM * m.nel / (el_ms_step * 1e-3) / 1e9 / hbm_peak_gbs()
                                  if hbm_peak_gbs() else None),
                     "hbm_bytes_per_elem": ALG_BYTES_PER_ELEM,
                     "fp64_equivalent_tflops": FLOP_PER_ELEM * m.nel / (el_ms_step * 1e-3) / 1e12,
                     "peak_source": f"instruction issue: 4 warp instructions per clock per SM x {nsm} SMs x "
                                    f"{sm_mhz:.0f} MHz (sampled); FP32 pipes, no FP64 peak applies"},
        "speedup_vs_plain_fp64": {"device": value / value64, "element_kernel": el64 / el_ms_step,
                                  "e2e": e2e64_s / e2e_s},
        "precision": precision,
        "plain_fp64": {
            "value": value64, "unit": UNIT, "ms_per_step": ms64, "element_kernel_ms": el64, "launches": launches64,
            "e2e": {"value": ws * m.nel / e2e64_s, "unit": UNIT, "ms_per_step": e2e64_s * 1e3},
            "roofline": {"bound": "fp64", "achieved": achieved64, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": achieved64 / fp64_peak, "traffic": traffic,
                         "kernel": "prism_elements_kernel", "kernel_ms": el64,
                         "flop_per_elem": FLOP_PER_ELEM, "fp64_pipe_slot_frac": slot_frac,
                         "textbook_flop_per_elem": TEXTBOOK_FLOP_PER_ELEM,
                         "peak_source": "FP64 FMA-chain kernel measured in this run (no FP64 figure in the peaks "
                                        "file)"}},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_s * 1e3,
                "note": "assembly tables cached on the device between calls (ModFEM keeps them from sir_create "
                        "to sir_free); e2e_cold uploads them in every call"},
        "e2e_cold": {"value": ws * m.nel / e2e_cold_s, "unit": UNIT, "h2d_bytes_per_step": h2d + table_bytes,
                     "d2h_bytes_per_step": d2h, "ms_per_step": e2e_cold_s * 1e3},
        "clocks": clocks,
        "solver": solver,
        "structure": structure,
        "dg": dg,
        "batch_mixed": batch,
        "serving": serving,
        "gpu_launches": launches,
        "wall_s_timed_region": wall,
    }
    if rank == 0:
        # the whole record to a file; one compact line (the figures the
        # headline rests on) to stdout
        try:
            d = os.path.dirname(DETAIL_FILE)
            if d:
                os.makedirs(d, exist_ok=True)
            with open(DETAIL_FILE, "w") as fh:
                json.dump(line, fh, indent=1)
        except OSError:
            pass
        print(json.dumps(compact_line(line)), flush=True)
    for pa in list(pins.values()) + [out_val, out_rhs]:
        pa.free()
    c.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
