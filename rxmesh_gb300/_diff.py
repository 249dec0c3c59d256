"""DiffScalarProblem mirror for the per-face ARAP term, and the torch autograd
bindings of the differentiable path.

DiffScalarProblem (include/rxmesh/diff/diff_scalar_problem.h:27-401) takes
user lambdas; lambdas cannot cross the C ABI, so the one energy of this path
(per-face ARAP against a flat rest frame) is a fixed term here:
`DiffScalarProblem(rx).add_arap_term(rest_xyz)` then `eval_terms(x)`.
"""
import ctypes

import torch

from . import _lib
from ._lib import check

_DT = {torch.float32: 0, torch.float64: 1}


def _stream(stream=None):
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class BlockSparseMatrix:
    """3x3-block CSR over the [diagonal, one-ring] pattern (HessianSparseMatrix)."""

    def __init__(self, n, nnzb, dtype, device):
        self.row_ptr = torch.zeros(n + 1, dtype=torch.int32, device=device)
        self.col = torch.zeros(nnzb, dtype=torch.int32, device=device)
        self.val = torch.zeros(nnzb, 3, 3, dtype=dtype, device=device)

    def to_csr(self, out=None, stream=None):
        """Scalar 3n x 3n CSR of this block matrix (rxg_bcsr_to_csr), the form
        the CG/PCG solvers take; out: a SparseMatrix of the right sizes to reuse."""
        from ._solvers import SparseMatrix
        n, nnzb = self.row_ptr.numel() - 1, self.col.numel()
        if out is None:
            dev = self.val.device
            out = SparseMatrix(row_ptr=torch.empty(3 * n + 1, dtype=torch.int32, device=dev),
                               col=torch.empty(9 * nnzb, dtype=torch.int32, device=dev),
                               val=torch.empty(9 * nnzb, dtype=self.val.dtype, device=dev))
        b, c = self.bcsr(), out.csr()
        check(_lib.load().rxg_bcsr_to_csr(ctypes.byref(b), ctypes.byref(c), _stream(stream)))
        return out

    def apply_bc(self, bc, grad=None, stream=None):
        """NewtonSolver::apply_bc (diff/newton_solver.h): bc (nv,) bool/int8 in
        linear order; identity diagonal blocks and zero coupling for
        constrained vertices, their gradient rows zeroed."""
        m = bc.to(torch.int8).contiguous()
        b = self.bcsr()
        check(_lib.load().rxg_bcsr_apply_bc(ctypes.byref(b), _p(m), _p(grad), _stream(stream)))

    def bcsr(self):
        b = _lib.BCSR()
        b.n = self.row_ptr.numel() - 1
        b.nnzb = self.col.numel()
        b.row_ptr = self.row_ptr.data_ptr()
        b.col = self.col.data_ptr()
        b.val = self.val.data_ptr()
        b.dtype = _DT[self.val.dtype]
        return b

    def to_scipy(self):
        import scipy.sparse as sp
        n = self.row_ptr.numel() - 1
        return sp.bsr_matrix((self.val.cpu().numpy(), self.col.cpu().numpy(),
                              self.row_ptr.cpu().numpy()), shape=(3 * n, 3 * n))


class DiffScalarProblem:
    """Energy / gradient / Hessian assembly driver (DiffScalarProblem<T,3,VertexHandle,true>)."""

    def __init__(self, rx, dtype=torch.float64, assemble_hessian=True):
        self.rx = rx
        self.dtype = dtype
        self.assemble_hessian = assemble_hessian
        self._L = _lib.load()
        dev = torch.device("cuda", torch.cuda.current_device())
        n, nnz = ctypes.c_int64(), ctypes.c_int64()
        check(self._L.rxg_mcf_pattern_size(rx._h, ctypes.byref(n), ctypes.byref(nnz)))
        self.grad = torch.zeros(n.value, 3, dtype=dtype, device=dev)
        self.face_energy = torch.zeros(rx.get_num_faces(), dtype=dtype, device=dev)
        self.hess = BlockSparseMatrix(n.value, nnz.value, dtype, dev) if assemble_hessian else None
        self.rest = None
        self.project_hessian = False
        self.opt_var = None
        self._loss = None

    def add_arap_term(self, rest_xyz_lin, project_hessian=False):
        """Per-face ARAP term against the flat rest frame of rest_xyz_lin (nv,3,
        linear order).  project_hessian: each face's 9x9 Hessian made positive
        definite before assembly (add_term<Op::FV, ProjectHess = true>)."""
        self.project_hessian = bool(project_hessian)
        xr = rest_xyz_lin.to(torch.float64).contiguous()
        self.rest = torch.empty(self.rx.get_num_faces(), 4, dtype=self.dtype, device=xr.device)
        check(self._L.rxg_arap_rest(self.rx._h, _p(xr), _DT[self.dtype], _p(self.rest), _stream()))
        return self

    def eval_terms(self, x_lin=None, with_hessian=None, stream=None):
        """Energy, gradient (and Hessian) at x_lin (nv,3, linear order), which
        becomes the problem's opt_var (x_lin None: at the current opt_var)."""
        if self.rest is None:
            raise RuntimeError("add_arap_term() first")
        if x_lin is not None:
            self.opt_var = x_lin
        x = self.opt_var.to(self.dtype).contiguous()
        h = self.assemble_hessian if with_hessian is None else with_hessian
        e = torch.zeros(1, dtype=torch.float64, device=x.device)
        b = self.hess.bcsr() if (h and self.hess is not None) else None
        check(self._L.rxg_arap_eval_ex(self.rx._h, _DT[self.dtype], _p(x), _p(self.rest),
                                       1 if self.project_hessian else 0, _p(e),
                                       _p(self.face_energy), _p(self.grad),
                                       ctypes.byref(b) if b is not None else None, _stream(stream)))
        self._loss = e
        return e

    def eval_terms_passive(self, x_lin, stream=None):
        """Energy alone at x_lin (eval_terms_passive, diff_scalar_problem.h):
        gradient, Hessian and opt_var are left untouched."""
        x = x_lin.to(self.dtype).contiguous()
        e = torch.zeros(1, dtype=torch.float64, device=x.device)
        check(self._L.rxg_arap_eval_ex(self.rx._h, _DT[self.dtype], _p(x), _p(self.rest), 0,
                                       _p(e), None, None, None, _stream(stream)))
        self._loss = e
        return e

    def eval_matvec(self, v, out=None, bc=None, stream=None):
        """out = H(opt_var) v without an assembled Hessian (eval_matvec,
        diff/diff_query_kernel.cuh:26-148; rxg_arap_hvp); bc (nv,) int8/bool:
        identity rows and zero columns for constrained vertices."""
        x = self.opt_var.to(self.dtype).contiguous()
        vv = v.to(self.dtype).contiguous()
        if out is None:
            out = torch.empty_like(vv)
        m = bc.to(torch.int8).contiguous() if bc is not None else None
        check(self._L.rxg_arap_hvp(self.rx._h, _DT[self.dtype], _p(x), _p(self.rest),
                                   1 if self.project_hessian else 0, _p(m), _p(vv), _p(out),
                                   _stream(stream)))
        return out

    def get_current_loss(self):
        return float(self._loss.item())


class NewtonSolver:
    """NewtonSolver<T, 3, VertexHandle, SolverT> (diff/newton_solver.h:17-330)
    on a DiffScalarProblem: compute_direction() solves H dir = -grad with a
    CG or PCG solver on the scalar form of the Hessian (rxg_bcsr_to_csr +
    rxg_cg_solve); line_search() backtracks on the energy with the Armijo
    test of diff/armijo_condition.h.  As in the reference, compute_direction
    leaves problem.grad negated, and the Armijo test then uses dir . grad of
    that negated gradient."""

    def __init__(self, problem, solver="pcg", max_iter=1000, abs_tol=1e-12, rel_tol=0.0):
        """solver: "pcg" or "cg" on the assembled Hessian's scalar form, or
        "cg_matfree" (CGMatFreeSolver: CG with Hessian-vector products from
        the face records, no assembled Hessian; rxg_arap_cg_matfree)."""
        from ._solvers import CGSolver, PCGSolver
        self.problem = problem
        self.dir = torch.zeros_like(problem.grad)
        self.matfree = solver == "cg_matfree"
        self._bc = None
        self._stats = _lib.SolverStats()
        self._solver_cls = PCGSolver if solver == "pcg" else CGSolver
        self.max_iter, self.abs_tol, self.rel_tol = max_iter, abs_tol, rel_tol
        self._A = None
        self.solver = None
        self.solve_time = 0.0

    def compute_direction(self, stream=None):
        p = self.problem
        p.grad.mul_(-1)
        if self.matfree:
            self.dir.zero_()
            x = p.opt_var.to(p.dtype).contiguous()
            o = _lib.SolverOpts(int(self.max_iter), float(self.abs_tol), float(self.rel_tol), 0)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            st = self._L().rxg_arap_cg_matfree(p.rx._h, _DT[p.dtype], _p(x), _p(p.rest),
                                              1 if p.project_hessian else 0, _p(self._bc),
                                              _p(p.grad), _p(self.dir), ctypes.byref(o),
                                              ctypes.byref(self._stats), _stream(stream))
            b.record()
            b.synchronize()
            if st not in (0, 6):
                check(st)
            self.solve_time += a.elapsed_time(b)
            return
        self._A = p.hess.to_csr(out=self._A, stream=stream)
        self.solver = self._solver_cls(self._A, 1, self.max_iter, self.abs_tol, self.rel_tol)
        self.dir.zero_()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        self.solver.solve(p.grad.reshape(-1, 1), self.dir.view(-1, 1), stream)
        b.record()
        b.synchronize()
        self.solve_time += a.elapsed_time(b)

    def line_search(self, s_max=1.0, shrink=0.8, max_iters=64, armijo_const=1e-4, cb=None,
                    stream=None):
        p = self.problem
        assert s_max > 0.0
        try_one = s_max > 1.0
        s = s_max
        f = p.get_current_loss()
        slope = float((self.dir * p.grad).sum())  # dir . grad, grad negated by compute_direction
        x = p.opt_var
        for _ in range(max_iters):
            t = x + s * self.dir.to(x.dtype)
            if cb is not None:
                cb(t)
            f_new = float(p.eval_terms_passive(t, stream).item())
            if f_new <= f + armijo_const * s * slope:
                x.copy_(t)
                return True
            if try_one and s > 1.0 and s * shrink < 1.0:
                s = 1.0
            else:
                s *= shrink
        return False

    def apply_bc(self, bc, stream=None):
        if self.matfree:
            # no assembled Hessian: the matrix-free products apply the
            # constraint; the gradient rows are zeroed here
            self._bc = bc.to(torch.int8).contiguous()
            keep = (self._bc == 0).to(self.problem.grad.dtype).unsqueeze(1)
            self.problem.grad.mul_(keep)
            return
        self.problem.hess.apply_bc(bc, self.problem.grad, stream)

    def iter_taken(self):
        return self._stats.iters if self.matfree else self.solver.iter_taken()

    @staticmethod
    def _L():
        return _lib.load()


def mcf_step_backward(rx, x_in, x_out, g_out, dt, tol=1e-12, max_iter=20000, stream=None):
    """dl/dx_in of one plain implicit MCF step, given dl/dx_out (rxg_mcf_step_backward)."""
    L = _lib.load()
    g_in = torch.empty_like(x_in)
    st = _lib.SolverStats()
    rc = L.rxg_mcf_step_backward(rx._h, float(dt), _p(x_in.contiguous()), _p(x_out.contiguous()),
                                 _p(g_out.contiguous()), _p(g_in), float(tol), int(max_iter),
                                 ctypes.byref(st), _stream(stream))
    if rc not in (0, 6):
        check(rc)
    return g_in


class ArapEnergy(torch.autograd.Function):
    """E = sum_f A_f ||J_f - R(J_f)||^2 at linear-order positions x (problem from DiffScalarProblem)."""

    @staticmethod
    def forward(ctx, x_lin, problem):
        e = problem.eval_terms(x_lin, with_hessian=False)
        ctx.save_for_backward(problem.grad.clone().to(x_lin.dtype))
        return e.to(x_lin.dtype).reshape(())

    @staticmethod
    def backward(ctx, go):
        (g,) = ctx.saved_tensors
        return go * g, None


class MCFFlow(torch.autograd.Function):
    """nsteps plain implicit MCF steps from x0 (linear order, FP64), differentiable in x0.

    The backward recomputes the flow segment by segment from positions saved
    every `checkpoint_every` steps (memory O(nsteps/k + k) states) and runs
    rxg_mcf_step_backward through each step in reverse."""

    @staticmethod
    def forward(ctx, x0_lin, rx, dt, nsteps, checkpoint_every=5, tol=1e-12, max_iter=20000):
        from ._solvers import mcf_step
        x = x0_lin.detach().to(torch.float64).contiguous().clone()
        ckpts = [x.clone()]
        for t in range(nsteps):
            mcf_step(rx, x, dt, 1, "f64", tol=tol, max_iter=max_iter)
            if (t + 1) % checkpoint_every == 0 and t + 1 < nsteps:
                ckpts.append(x.clone())
        ctx.rx, ctx.dt, ctx.nsteps, ctx.k = rx, dt, nsteps, checkpoint_every
        ctx.tol, ctx.max_iter = tol, max_iter
        ctx.save_for_backward(*ckpts)
        return x

    @staticmethod
    def backward(ctx, g):
        from ._solvers import mcf_step
        ckpts = ctx.saved_tensors
        g = g.to(torch.float64).contiguous()
        k, n = ctx.k, ctx.nsteps
        for seg in reversed(range(len(ckpts))):
            start = seg * k
            end = min(start + k, n)
            states = [ckpts[seg]]
            for _ in range(start, end):
                x = states[-1].clone()
                mcf_step(ctx.rx, x, ctx.dt, 1, "f64", tol=ctx.tol, max_iter=ctx.max_iter)
                states.append(x)
            for t in reversed(range(end - start)):
                g = mcf_step_backward(ctx.rx, states[t], states[t + 1], g, ctx.dt, ctx.tol, ctx.max_iter)
        return g, None, None, None, None, None, None


def mcf_flow(x0_lin, rx, dt, nsteps, checkpoint_every=5, tol=1e-12, max_iter=20000):
    return MCFFlow.apply(x0_lin, rx, dt, nsteps, checkpoint_every, tol, max_iter)


def arap_energy(x_lin, problem):
    return ArapEnergy.apply(x_lin, problem)
