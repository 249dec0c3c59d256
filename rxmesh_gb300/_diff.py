"""DiffScalarProblem mirror and the torch autograd bindings of the
differentiable path.

DiffScalarProblem (include/rxmesh/diff/diff_scalar_problem.h:27-401) takes
user lambdas over a forward-mode Scalar; lambdas cannot cross the C ABI, so
from Python the terms are the library's built-in per-face energies:
`add_arap_term(rest_xyz)` (3 components per vertex) and
`add_symmetric_dirichlet_term(rest_xyz)` (Param's energy on 2-D uv), each
evaluated through the forward-mode Scalar type of include/rxg/diff.cuh or
its closed form, and summed by eval_terms(x).  C++ applications write their
own terms with include/rxg/diff.cuh and rxg_face_term_gather /
rxg_edge_term_gather / rxg_vertex_term_gather; from Python, add_term(op, fn)
takes a function that returns the per-element records (energy, gradient,
packed Hessian) of a term, which the library assembles.
"""
import ctypes

import torch

from . import _lib
from ._lib import check

_DT = {torch.float32: 0, torch.float64: 1}
RXG_TERM_ACCUMULATE = 1
RXG_TERM_PROJECT_HESSIAN = 2


def _stream(stream=None):
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class BlockSparseMatrix:
    """D x D-block CSR over the [diagonal, one-ring] pattern
    (HessianSparseMatrix<T, D>); D = dim, 3 by default."""

    def __init__(self, n, nnzb, dtype, device, dim=3):
        self.dim = int(dim)
        self.row_ptr = torch.zeros(n + 1, dtype=torch.int32, device=device)
        self.col = torch.zeros(nnzb, dtype=torch.int32, device=device)
        self.val = torch.zeros(nnzb, self.dim, self.dim, dtype=dtype, device=device)

    def to_csr(self, out=None, stream=None):
        """Scalar (D n) x (D n) CSR of this block matrix (rxg_bcsr_to_csr), the
        form the CG/PCG solvers take; out: a SparseMatrix of the right sizes to reuse."""
        from ._solvers import SparseMatrix
        n, nnzb, d = self.row_ptr.numel() - 1, self.col.numel(), self.dim
        if out is None:
            dev = self.val.device
            out = SparseMatrix(row_ptr=torch.empty(d * n + 1, dtype=torch.int32, device=dev),
                               col=torch.empty(d * d * nnzb, dtype=torch.int32, device=dev),
                               val=torch.empty(d * d * nnzb, dtype=self.val.dtype, device=dev))
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
        b.block_dim = self.dim
        return b

    def to_scipy(self):
        import scipy.sparse as sp
        n, d = self.row_ptr.numel() - 1, self.dim
        return sp.bsr_matrix((self.val.cpu().numpy(), self.col.cpu().numpy(),
                              self.row_ptr.cpu().numpy()), shape=(d * n, d * n))


class DiffScalarProblem:
    """Energy / gradient / Hessian assembly driver
    (DiffScalarProblem<T, dim, VertexHandle, true>): the sum of its terms.

    dim: components of the optimisation variable per vertex (3 for the ARAP
    term on positions, 2 for the symmetric Dirichlet term on uv)."""

    def __init__(self, rx, dtype=torch.float64, assemble_hessian=True, dim=3):
        self.rx = rx
        self.dtype = dtype
        self.dim = int(dim)
        self.assemble_hessian = assemble_hessian
        self._L = _lib.load()
        dev = torch.device("cuda", torch.cuda.current_device())
        n, nnz = ctypes.c_int64(), ctypes.c_int64()
        check(self._L.rxg_mcf_pattern_size(rx._h, ctypes.byref(n), ctypes.byref(nnz)))
        self.grad = torch.zeros(n.value, self.dim, dtype=dtype, device=dev)
        self.face_energy = torch.zeros(rx.get_num_faces(), dtype=dtype, device=dev)
        self.hess = (BlockSparseMatrix(n.value, nnz.value, dtype, dev, self.dim)
                     if assemble_hessian else None)
        self.terms = []  # (kind, rest frames Mr^-1 (nf, 4) or target positions, project or mass)
        self.rest = None
        self.project_hessian = False
        self.opt_var = None
        self._loss = None
        self._tmp_face = None

    def _rest_frames(self, rest_xyz_lin):
        xr = rest_xyz_lin.to(torch.float64).contiguous()
        rest = torch.empty(self.rx.get_num_faces(), 4, dtype=self.dtype, device=xr.device)
        check(self._L.rxg_arap_rest(self.rx._h, _p(xr), _DT[self.dtype], _p(rest), _stream()))
        return rest

    def add_arap_term(self, rest_xyz_lin, project_hessian=False):
        """Per-face ARAP term against the flat rest frame of rest_xyz_lin (nv,3,
        linear order).  project_hessian: each face's 9x9 Hessian made positive
        definite before assembly (add_term<Op::FV, ProjectHess = true>).
        Needs dim = 3 and comes first among the terms."""
        if self.dim != 3 or self.terms:
            raise ValueError("the ARAP term needs dim=3 and is the problem's first term")
        self.project_hessian = bool(project_hessian)
        self.rest = self._rest_frames(rest_xyz_lin)
        self.terms.append(("arap", self.rest, self.project_hessian))
        return self

    def add_symmetric_dirichlet_term(self, rest_xyz_lin, project_hessian=False):
        """Param's symmetric Dirichlet energy (apps/Param/param.cu:146-183) of
        the uv parameterisation (opt_var (nv,2)): per face A (|J|^2 +
        |J^-1|^2), J = M Mr^-1 with Mr the face's rest shape in its own plane
        (rest_xyz_lin (nv,3), linear order).  Needs dim = 2."""
        if self.dim != 2:
            raise ValueError("the symmetric Dirichlet term needs dim=2 (uv)")
        rest = self._rest_frames(rest_xyz_lin)
        if self.rest is None:
            self.rest = rest
        self.terms.append(("symdir", rest, bool(project_hessian)))
        return self

    def add_inertia_term(self, x_target_lin, mass):
        """Inertia of a mass-spring system (add_inertia_term,
        tests/RXMesh_test/test_hess.cu:13-29): per vertex mass/2 |x - x_target|^2,
        Hessian mass I.  x_target_lin (nv, dim), linear order."""
        xt = x_target_lin.to(self.dtype).contiguous().clone()
        self.terms.append(("inertia", xt, float(mass)))
        return self

    def add_term(self, op, records_fn):
        """A term given by its per-element records (add_term<Op::FV / Op::EV /
        Op::V>, diff_scalar_problem.h:127-194): records_fn(x) for x (nv, dim)
        in linear order returns an (n, W) tensor of the problem's dtype on
        x's device, one row per face / edge / vertex in linear order, W = 1 +
        K + K (K + 1) / 2 with K = c * dim and c = 3, 2, 1: the element's
        energy, its gradient (the element's vertices in FV / EV order, dim
        components each) and the upper triangle of its K x K Hessian, row by
        row.  The library assembles the gradient and the block Hessian."""
        op = str(op).upper()
        if op not in ("FV", "EV", "V"):
            raise ValueError("terms are per face (FV), edge (EV) or vertex (V)")
        self.terms.append(("rec_" + op.lower(), records_fn, False))
        return self

    def _records_term(self, kind, fn, x, i, e, fe, grad, hb, stream):
        c = {"rec_fv": 3, "rec_ev": 2, "rec_v": 1}[kind]
        n = {"rec_fv": self.rx.get_num_faces(), "rec_ev": self.rx.get_num_edges(),
             "rec_v": self.rx.get_num_vertices()}[kind]
        k = c * self.dim
        rec = fn(x)
        if rec.dtype != self.dtype or rec.device != x.device or tuple(rec.shape) != (n, 1 + k + k * (k + 1) // 2):
            raise ValueError(f"term records: want ({n}, {1 + k + k * (k + 1) // 2}) {self.dtype} on {x.device}, "
                             f"got {tuple(rec.shape)} {rec.dtype} on {rec.device}")
        rec = rec.contiguous()
        fn_c = {"rec_fv": self._L.rxg_face_term_gather, "rec_ev": self._L.rxg_edge_term_gather,
                "rec_v": self._L.rxg_vertex_term_gather}[kind]
        check(fn_c(self.rx._h, _DT[self.dtype], self.dim, _p(rec), RXG_TERM_ACCUMULATE if i > 0 else 0,
                   _p(e), _p(fe) if kind == "rec_fv" else None, _p(grad), hb, _stream(stream)))

    def _eval(self, x, grad, face_E, hess_b, with_projection=True, stream=None):
        """Sum of the terms at x; returns the energy (1-element FP64 tensor)."""
        if not self.terms:
            raise RuntimeError("add a term first")
        total = torch.zeros(1, dtype=torch.float64, device=x.device)
        for i, (kind, rest, proj) in enumerate(self.terms):
            e = torch.zeros(1, dtype=torch.float64, device=x.device)
            fe = face_E
            if fe is not None and i > 0:
                if self._tmp_face is None:
                    self._tmp_face = torch.empty_like(self.face_energy)
                fe = self._tmp_face
            hb = ctypes.byref(hess_b) if hess_b is not None else None
            pj = proj and with_projection
            if kind.startswith("rec_"):
                self._records_term(kind, rest, x, i, e, fe, grad, hb, stream)
                if kind != "rec_fv" and face_E is not None and i == 0:
                    face_E.zero_()
                if kind == "rec_fv" and fe is not None and i > 0:
                    face_E.add_(fe)
                total += e
                continue
            if kind == "inertia":
                check(self._L.rxg_inertia_eval(self.rx._h, _DT[self.dtype], self.dim, _p(x), _p(rest),
                                               ctypes.c_double(proj), RXG_TERM_ACCUMULATE if i > 0 else 0,
                                               _p(e), _p(grad), hb, _stream(stream)))
                if face_E is not None and i == 0:
                    face_E.zero_()
                total += e
                continue
            if kind == "arap":
                check(self._L.rxg_arap_eval_ex(self.rx._h, _DT[self.dtype], _p(x), _p(rest),
                                               1 if pj else 0, _p(e), _p(fe), _p(grad), hb,
                                               _stream(stream)))
            else:
                flags = (RXG_TERM_ACCUMULATE if i > 0 else 0) | (RXG_TERM_PROJECT_HESSIAN if pj else 0)
                check(self._L.rxg_symdir_eval(self.rx._h, _DT[self.dtype], _p(x), _p(rest), flags,
                                              _p(e), _p(fe), _p(grad), hb, _stream(stream)))
            if fe is not None and i > 0:
                face_E.add_(fe)
            total += e
        return total

    def eval_terms(self, x_lin=None, with_hessian=None, stream=None):
        """Energy, gradient (and Hessian) at x_lin (nv, dim, linear order),
        which becomes the problem's opt_var (x_lin None: at the current opt_var)."""
        if x_lin is not None:
            self.opt_var = x_lin
        x = self.opt_var.to(self.dtype).contiguous()
        h = self.assemble_hessian if with_hessian is None else with_hessian
        b = self.hess.bcsr() if (h and self.hess is not None) else None
        self._loss = self._eval(x, self.grad, self.face_energy, b, stream=stream)
        return self._loss

    def eval_terms_passive(self, x_lin, stream=None):
        """Energy alone at x_lin (eval_terms_passive, diff_scalar_problem.h):
        gradient, Hessian and opt_var are left untouched."""
        x = x_lin.to(self.dtype).contiguous()
        self._loss = self._eval(x, None, None, None, with_projection=False, stream=stream)
        return self._loss

    def eval_matvec(self, v, out=None, bc=None, stream=None):
        """out = H(opt_var) v (eval_matvec, diff/diff_query_kernel.cuh:26-148):
        for the ARAP term without an assembled Hessian (rxg_arap_hvp); for
        the other terms through the assembled Hessian's scalar form.  bc
        (nv,) int8/bool: identity rows and zero columns for constrained
        vertices."""
        x = self.opt_var.to(self.dtype).contiguous()
        vv = v.to(self.dtype).contiguous()
        if out is None:
            out = torch.empty_like(vv)
        m = bc.to(torch.int8).contiguous() if bc is not None else None
        if len(self.terms) == 1 and self.terms[0][0] == "arap":
            check(self._L.rxg_arap_hvp(self.rx._h, _DT[self.dtype], _p(x), _p(self.rest),
                                       1 if self.project_hessian else 0, _p(m), _p(vv), _p(out),
                                       _stream(stream)))
            return out
        H = self.hess
        if H is None:
            nn, nz = ctypes.c_int64(), ctypes.c_int64()
            check(self._L.rxg_mcf_pattern_size(self.rx._h, ctypes.byref(nn), ctypes.byref(nz)))
            H = BlockSparseMatrix(nn.value, nz.value, self.dtype, x.device, self.dim)
        self._eval(x, torch.empty_like(self.grad), None, H.bcsr(), stream=stream)
        if m is not None:
            H.apply_bc(m, None, stream)
        H.to_csr(stream=stream).multiply(vv.reshape(-1, 1), out.view(-1, 1), stream)
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
