"""Optional torch binding: a batch of conic QPs as a differentiable layer.

QPLayer holds a BatchSolver whose sparsity patterns are fixed at construction; forward(Px, q,
Ax, b) takes the concatenated values of every instance as CUDA float64 tensors, solves the whole
batch on the tensor's current stream and returns the concatenated primal solutions x. Backward
runs the adjoint kernel (one extra KKT solve per instance with the saved final factorisation)
and returns gradients for all four value tensors. No copy leaves the device.
"""
import torch

from . import _abi
from .solver import BatchSolver


class _QPFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, Px, q, Ax, b, solver):
        for t in (Px, q, Ax, b):
            if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
                raise ValueError("QPLayer inputs must be contiguous CUDA float64 tensors")
        stream = torch.cuda.current_stream(Px.device).cuda_stream
        x = torch.empty(solver.n_total, dtype=torch.float64, device=Px.device)
        s = torch.empty(solver.m_total, dtype=torch.float64, device=Px.device)
        z = torch.empty(solver.m_total, dtype=torch.float64, device=Px.device)
        solver.update_values_device(Px.data_ptr(), q.data_ptr(), Ax.data_ptr(), b.data_ptr(), stream)
        solver.solve_device(x.data_ptr(), s.data_ptr(), z.data_ptr(), stream)
        ctx.solver = solver
        ctx.mark_non_differentiable(s, z)
        return x, s, z

    @staticmethod
    def backward(ctx, gx, gs, gz):
        solver = ctx.solver
        gx = gx.contiguous()
        dev = gx.device
        stream = torch.cuda.current_stream(dev).cuda_stream
        dq = torch.empty(solver.n_total, dtype=torch.float64, device=dev)
        db = torch.empty(solver.m_total, dtype=torch.float64, device=dev)
        dP = torch.empty(solver.nnzP, dtype=torch.float64, device=dev)
        dA = torch.empty(solver.nnzA, dtype=torch.float64, device=dev)
        solver.backward_device(gx.data_ptr(), dq.data_ptr(), db.data_ptr(), dP.data_ptr(), dA.data_ptr(), stream)
        return dP, dq, dA, db, None


class QPLayer(torch.nn.Module):
    """x = argmin 1/2 x'Px + q'x s.t. Ax + s = b, s in K, for every instance of a batch.

    `qps` fixes the batch (sizes, cone specs, sparsity patterns, equilibration); the values are
    the forward arguments. Mixed precision by default (settings may override)."""

    def __init__(self, qps, settings=None, **kw):
        super().__init__()
        kw.setdefault("differentiable", 1)
        kw.setdefault("warm_start", 0)
        if settings is None:
            settings = _abi.default_settings(precision=_abi.PRECISION_MIXED)
        self.solver = BatchSolver(qps, settings=settings, **kw)

    def forward(self, Px, q, Ax, b):
        x, s, z = _QPFunction.apply(Px, q, Ax, b, self.solver)
        return x

    def split(self, x):
        """Per-instance views of a concatenated solution tensor."""
        o = self.solver.n_off
        return [x[o[i]:o[i + 1]] for i in range(self.solver.count)]
