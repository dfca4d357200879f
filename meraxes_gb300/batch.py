"""A batch of independent boxes (seeds, parameter draws and box sizes) with
the forward step and the adjoint of the power-spectrum loss for each.

Each box is one snapshot of the differentiation workload's physics (the full
step at z=12: ComputeTs, find_HII_bubbles with recombinations, the 21cm box)
at its own size, seed, L_X and escape fraction.  Boxes of one size share a
grid layout, so a worker (a host thread with its own library context and CUDA
stream) runs the boxes of one size one after another; workers of all sizes
run at the same time and their kernels overlap on the GPU.  The packing -- how
many workers each size gets -- comes from the measured device memory of one
context per size: as many as fit in the free memory, up to the number of boxes
and a cap.  Results do not depend on the packing: every box's arithmetic is the
same whichever worker runs it.
"""
from __future__ import annotations

import dataclasses
import math
import threading
import time
from typing import Dict, List, Optional, Sequence

import numpy as np

from .params import ReionParams, Workload, workload


@dataclasses.dataclass
class Instance:
    grid_dim: int
    seed: int
    lx_gal: float
    fesc: float
    cell: float = 0.5  # Mpc/h


def uneven_batch(n_per_size: int = 16, sizes: Sequence[int] = (96, 128, 192), seed0: int = 10,
                 draw_seed: int = 2024) -> List[Instance]:
    """The uneven batch: n_per_size boxes at each size with 0.5 Mpc/h cells,
    seeds seed0, seed0 + 1, ..., and (log10 L_X, escape fraction) drawn
    uniformly from [39, 41] x [0.05, 0.3] with a fixed generator."""
    rng = np.random.default_rng(draw_seed)
    out = []
    seed = seed0
    for D in sizes:
        for _ in range(n_per_size):
            lx = 10.0 ** rng.uniform(39.0, 41.0)
            out.append(Instance(D, seed, float(lx), float(rng.uniform(0.05, 0.3))))
            seed += 1
    return out


def instance_workload(inst: Instance) -> Workload:
    base = workload("diff_256")
    p = dataclasses.replace(base.params, grid_dim=inst.grid_dim, box_size=inst.cell * inst.grid_dim,
                            lx_gal=inst.lx_gal)
    w = Workload(f"box{inst.grid_dim}_s{inst.seed}", p, inst.seed, list(base.redshifts), list(base.snapshots))
    w.fesc = 1.0  # the escape fraction multiplies the stars grid in the differentiable forward
    return w


class _Prepared:
    """Device inputs and the loss target of one box."""

    def __init__(self, inst: Instance, n_hist: int, target_lx: float, step):
        import torch

        from . import synthetic as syn
        from .autograd import DeltaT21, log_bins

        self.inst = inst
        w = instance_workload(inst)
        self.w = w
        st = syn.initial_state(w.params, w.redshifts[0])
        st.update(syn.FieldGenerator(w).inputs(1, n_hist))
        D = w.params.grid_dim
        st.setdefault("delta_T", np.zeros((D, D, D), np.float32))
        self.dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in st.items()}
        self.state = {k: v for k, v in self.dev.items() if k not in ("sfr", "stars")}
        self.edges = log_bins(step, 20)
        with torch.no_grad():
            dT = DeltaT21.apply(self.dev["sfr"], self.dev["stars"] * inst.fesc,
                                torch.tensor(target_lx, dtype=torch.float64),
                                torch.tensor(w.params.nu_xray_gal_threshold, dtype=torch.float64), step, 1,
                                self.state)
            _, self.target, _ = step.ps_loss(dT, self.edges, [0.0] * 20, grad=False)


class BatchRunner:
    def __init__(self, instances: Sequence[Instance], target_lx: float = 2e40, max_workers_per_size: int = 4,
                 memory_fraction: float = 0.8, log: bool = False):
        self.log = log
        self.instances = list(instances)
        self.target_lx = target_lx
        self.max_workers = max_workers_per_size
        self.memory_fraction = memory_fraction
        self.sizes = sorted({i.grid_dim for i in self.instances})
        self.plan: Dict[int, int] = {}
        self.ctx_bytes: Dict[int, int] = {}

    def _new_step(self, D: int):
        from .api import ReionGridStep

        inst = next(i for i in self.instances if i.grid_dim == D)
        w = instance_workload(inst)
        # transform batches of 5 radii x 5 fields: enough for small boxes
        return ReionGridStep(w.params, w.redshifts, max_work_bytes=25 * 8 * D * D * (D // 2 + 16))

    def make_plan(self) -> Dict[int, int]:
        """Workers per size: the device memory of one context per size,
        measured, and as many workers as fit in memory_fraction of the free
        memory, split evenly over the sizes, up to the boxes of that size and
        max_workers_per_size."""
        import torch

        steps = {}
        for D in self.sizes:
            torch.cuda.synchronize()
            free0, _ = torch.cuda.mem_get_info()
            steps[D] = self._new_step(D)
            torch.cuda.synchronize()
            free1, _ = torch.cuda.mem_get_info()
            # context + this size's box inputs and the step's copies (about 40 grids)
            self.ctx_bytes[D] = (free0 - free1) + 40 * 4 * D ** 3
        free, _ = torch.cuda.mem_get_info()
        budget = self.memory_fraction * free / max(len(self.sizes), 1)
        for D in self.sizes:
            n = sum(1 for i in self.instances if i.grid_dim == D)
            self.plan[D] = int(max(1, min(n, self.max_workers, budget // max(self.ctx_bytes[D], 1))))
        self._probe_steps = steps
        return self.plan

    def run(self) -> Dict[str, object]:
        """Forward + adjoint of every box.  Returns per-box losses and
        gradients (in instance order) and the wall time of the timed part
        (inputs and targets are prepared before it)."""
        import torch

        from .autograd import DeltaT21, PSLoss21

        if not self.plan:
            self.make_plan()
        # workers: one context each (the planning contexts are reused)
        workers = []
        for D in self.sizes:
            for k in range(self.plan[D]):
                step = self._probe_steps.pop(D) if k == 0 and D in self._probe_steps else self._new_step(D)
                workers.append((D, step))
        queues = {id(s): [] for _, s in workers}
        by_size: Dict[int, List] = {}
        for D, s in workers:
            by_size.setdefault(D, []).append(s)
        for idx, inst in enumerate(self.instances):
            ws = by_size[inst.grid_dim]
            queues[id(ws[len([1 for j in self.instances[:idx] if j.grid_dim == inst.grid_dim]) % len(ws)])].append(idx)
        prepared: Dict[int, _Prepared] = {}
        for D, s in workers:
            for idx in queues[id(s)]:
                if self.log:
                    print(f"prepare box {idx} D={D}", flush=True)
                prepared[idx] = _Prepared(self.instances[idx], s.n_sfr_histories, self.target_lx, s)
        torch.cuda.synchronize()
        results: List[Optional[dict]] = [None] * len(self.instances)
        errors = []

        def work(step, idxs):
            try:
                stream = torch.cuda.Stream()
                with torch.cuda.stream(stream):
                    for idx in idxs:
                        pr = prepared[idx]
                        inst = pr.inst
                        if self.log:
                            print(f"box {idx} D={inst.grid_dim} start", flush=True)
                        sfr = pr.dev["sfr"].clone().requires_grad_(True)
                        fesc = torch.tensor(inst.fesc, device="cuda", requires_grad=True)
                        lx = torch.tensor(inst.lx_gal, dtype=torch.float64, requires_grad=True)
                        e0 = torch.tensor(pr.w.params.nu_xray_gal_threshold, dtype=torch.float64,
                                          requires_grad=True)
                        L = PSLoss21.apply(DeltaT21.apply(sfr, pr.dev["stars"] * fesc, lx, e0, step, 1, pr.state),
                                           step, pr.edges, pr.target)
                        L.backward()
                        stream.synchronize()
                        results[idx] = {"grid_dim": inst.grid_dim, "seed": inst.seed, "loss": L.item(),
                                        "dL_dLX": lx.grad.item(), "dL_dE0": e0.grad.item(),
                                        "dL_dfesc": fesc.grad.item(),
                                        "dL_dsfr_sum": float(sfr.grad.double().sum().item())}
            except Exception as e:  # noqa: BLE001
                errors.append(e)

        threads = [threading.Thread(target=work, args=(s, queues[id(s)])) for _, s in workers]
        t0 = time.perf_counter()
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        if errors:
            raise errors[0]
        return {"results": results, "wall_s": wall, "plan": dict(self.plan),
                "ctx_bytes": {int(k): int(v) for k, v in self.ctx_bytes.items()}}


__all__ = ["Instance", "uneven_batch", "instance_workload", "BatchRunner"]
