"""Host-side mirror of the reference's partial-assembly interface for this
path (same class and method names as MFEM, same argument meaning and error
behaviour), driving the CUDA library through its C ABI. Device memory is held
in torch tensors; torch is plumbing here, every computation on the path is a
libgbpa kernel.

    dev = Device("cuda")
    fes = FiniteElementSpace(CartesianMesh(8), p=3)
    a = BilinearForm(fes)
    a.AddDomainIntegrator(DiffusionIntegrator(ir_points=4))
    a.SetAssemblyLevel(AssemblyLevel.PARTIAL)
    a.Assemble()
    A, X, B = a.FormLinearSystem(ess_tdof_list, x, b)
    M = OperatorJacobiSmoother(a, ess_tdof_list)
    cg = CGSolver(); cg.SetRelTol(1e-12); cg.SetMaxIter(500)
    cg.SetOperator(A); cg.SetPreconditioner(M); cg.Mult(B, X)
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .fem import H1Space, Tables

check = _lib.check


def _p(t):
    """Device pointer of a tensor (or None)."""
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class AssemblyLevel:
    LEGACY, FULL, ELEMENT, PARTIAL, NONE = range(5)


class Device:
    """mfem::Device("cuda"): owns the library context on one GPU."""
    _current = None

    def __init__(self, spec="cuda", device_id=0):
        if spec not in ("cuda", "gpu"):
            raise ValueError("only the CUDA device is provided by this library")
        if not torch.cuda.is_available():
            raise RuntimeError("Device('cuda') requires a CUDA GPU")
        self.lib = _lib.load()
        torch.cuda.set_device(device_id)
        self.torch_device = torch.device("cuda", device_id)
        h = ctypes.c_void_p()
        check(self.lib.gbpa_create(ctypes.byref(h), device_id), "gbpa_create")
        self.ctx = h
        # run on torch's current stream so torch-side copies are ordered with
        # ours; torch's default stream has handle 0, which the library reads as
        # "own stream", so name the legacy default stream (handle 1) instead
        h = torch.cuda.current_stream().cuda_stream
        check(self.lib.gbpa_set_stream(self.ctx, ctypes.c_void_p(h if h else 1)), "gbpa_set_stream")
        # block shapes chosen by the autotuner (mfem_gb300/tuning.json), if present
        from .autotune import load_default
        self.tuned_entries = load_default(self.lib)
        Device._current = self

    @classmethod
    def get(cls):
        if cls._current is None:
            cls._current = Device("cuda")
        return cls._current

    def launches(self):
        return self.lib.gbpa_launch_count(self.ctx)

    def synchronize(self):
        check(self.lib.gbpa_synchronize(self.ctx), "gbpa_synchronize")

    def error_flags(self):
        f = ctypes.c_int(0)
        check(self.lib.gbpa_get_error_flags(self.ctx, ctypes.byref(f)), "gbpa_get_error_flags")
        return f.value

    def __del__(self):
        try:
            if self.ctx:
                self.lib.gbpa_destroy(self.ctx)
        except Exception:
            pass


def _dev():
    return Device.get()


def to_dev(a, dtype=None):
    d = _dev().torch_device
    if isinstance(a, torch.Tensor):
        return a.to(device=d, dtype=dtype or a.dtype).contiguous()
    a = np.ascontiguousarray(a)
    t = torch.from_numpy(a)
    return t.to(device=d, dtype=dtype or t.dtype).contiguous()


class ElementRestriction:
    """fem/restriction.cpp ElementRestriction (LEXICOGRAPHIC, vdim 1)."""

    def __init__(self, ne, dof, ndofs, elem_dofs, dof_map=None, build_on_device=False):
        self.ne, self.dof, self.ndofs = ne, dof, ndofs
        lib = _dev().lib
        if build_on_device:
            ed = to_dev(np.asarray(elem_dofs, np.int32))
            dm = to_dev(np.asarray(dof_map, np.int32)) if dof_map is not None else None
            d = _dev().torch_device
            self.offsets = torch.empty(ndofs + 1, dtype=torch.int32, device=d)
            self.indices = torch.empty(ne * dof, dtype=torch.int32, device=d)
            self.gather_map = torch.empty(ne * dof, dtype=torch.int32, device=d)
            check(lib.gbpa_restriction_build_device(_dev().ctx, ne, dof, ndofs, _p(ed), _p(dm),
                                                    _p(self.offsets), _p(self.indices),
                                                    _p(self.gather_map)), "restriction_build_device")
        else:
            ed = np.ascontiguousarray(elem_dofs, np.int32)
            dm = None if dof_map is None else np.ascontiguousarray(dof_map, np.int32)
            off = np.zeros(ndofs + 1, np.int32)
            ind = np.zeros(ne * dof, np.int32)
            gm = np.zeros(ne * dof, np.int32)
            check(lib.gbpa_restriction_build(ne, dof, ndofs, ed.ctypes.data_as(ctypes.c_void_p),
                                             None if dm is None else dm.ctypes.data_as(ctypes.c_void_p),
                                             off.ctypes.data_as(ctypes.c_void_p),
                                             ind.ctypes.data_as(ctypes.c_void_p),
                                             gm.ctypes.data_as(ctypes.c_void_p)), "restriction_build")
            self.offsets, self.indices, self.gather_map = to_dev(off), to_dev(ind), to_dev(gm)

    @classmethod
    def from_maps(cls, ne, dof, ndofs, gather_map, offsets, indices):
        r = cls.__new__(cls)
        r.ne, r.dof, r.ndofs = ne, dof, ndofs
        r.gather_map, r.offsets, r.indices = to_dev(gather_map), to_dev(offsets), to_dev(indices)
        return r

    def Mult(self, x, y):
        check(_dev().lib.gbpa_restriction_mult(_dev().ctx, self.ne, self.dof, 1, 0, self.ndofs,
                                               _p(self.gather_map), _p(x), _p(y)), "restriction_mult")

    def MultTranspose(self, x, y):
        check(_dev().lib.gbpa_restriction_mult_transpose(_dev().ctx, self.ne, self.dof, 1, 0, self.ndofs,
                                                         _p(self.offsets), _p(self.indices), _p(x),
                                                         _p(y), 0), "restriction_mult_transpose")

    def AddMultTranspose(self, x, y):
        check(_dev().lib.gbpa_restriction_mult_transpose(_dev().ctx, self.ne, self.dof, 1, 0, self.ndofs,
                                                         _p(self.offsets), _p(self.indices), _p(x),
                                                         _p(y), 1), "restriction_add_mult_transpose")

    def AbsMultTranspose(self, x, y):
        check(_dev().lib.gbpa_restriction_abs_mult_transpose(_dev().ctx, self.ne, self.dof, 1, 0,
                                                             self.ndofs, _p(self.offsets),
                                                             _p(self.indices), _p(x), _p(y)),
              "restriction_abs_mult_transpose")


class FiniteElementSpace:
    """H1 order-p space on a CartesianMesh (global lexicographic numbering)."""

    def __init__(self, mesh, p):
        self.mesh, self.p = mesh, p
        self.space = H1Space(mesh, p)
        self.ndofs = self.space.ndofs
        self.ne = mesh.ne
        self._restriction = None

    def GetNDofs(self):
        return self.ndofs

    def GetTrueVSize(self):
        return self.ndofs

    def GetNE(self):
        return self.ne

    def GetElementRestriction(self):
        if self._restriction is None:
            self._restriction = ElementRestriction(self.ne, (self.p + 1) ** 3, self.ndofs,
                                                   self.space.element_dofs(), None)
        return self._restriction

    def GetBoundaryTrueDofs(self):
        return self.space.boundary_dofs()


class _PAIntegrator:
    kind = None

    def __init__(self, coeff=None, ir_points=None):
        # coeff: None (1), float (constant), "kappa" (lognormal field at the
        # quadrature points), or a callable f(xyz torch (..., 3)) -> values
        self.coeff = coeff
        self.ir_points = ir_points

    def quad_points(self, p):
        return self.ir_points if self.ir_points else p + 2

    def _coefficient(self, fes, tables, geom):
        dev = _dev()
        c = self.coeff
        if c is None or isinstance(c, (int, float)):
            return to_dev(np.array([1.0 if c is None else float(c)])), 1
        # non-constant: evaluate at the physical quadrature points on the device
        ne, Q = fes.ne, tables.Q
        XQ = torch.empty(Q ** 3 * 3 * ne, dtype=torch.float64, device=dev.torch_device)
        check(dev.lib.gbpa_geom_coordinates3d(dev.ctx, ne, geom["dg"], Q, _p(geom["Bg"]),
                                              _p(geom["X"]), _p(XQ)), "geom_coordinates3d")
        if c == "kappa":
            # the lognormal field, evaluated by the library's kernel
            k, phi = geom["modes"]
            kk = np.ascontiguousarray(k, dtype=np.int32).reshape(-1)
            ph = np.ascontiguousarray(phi, dtype=np.float64)
            vals = torch.empty(Q ** 3 * ne, dtype=torch.float64, device=dev.torch_device)
            check(dev.lib.gbpa_coefficient_lognormal3d(
                dev.ctx, ne, Q ** 3, _p(XQ), len(ph), kk.ctypes.data_as(ctypes.c_void_p),
                ph.ctypes.data_as(ctypes.c_void_p), 0.5, _p(vals)), "coefficient_lognormal3d")
            return vals, 1
        # a user function of the coordinates, evaluated by torch on the device
        xyz = XQ.view(ne, 3, Q ** 3).permute(0, 2, 1)
        return c(xyz).contiguous().view(-1), 1


def _geometry(fes, tables, modes):
    mesh = fes.mesh
    order = 3 if mesh.curved else 1
    dg = order + 1
    gt = Tables(order, tables.Q)
    X = to_dev(mesh.nodes_evector(order))
    return {"dg": dg, "Bg": to_dev(gt.B), "Gg": to_dev(gt.G), "X": X, "modes": modes}


class DiffusionIntegrator(_PAIntegrator):
    kind = _lib.GBPA_DIFFUSION

    def AssemblePA(self, fes, modes=None):
        dev = _dev()
        p = fes.p
        self.tables = t = Tables(p, self.quad_points(p))
        self.fes = fes
        self.D, self.Q, self.ne = t.D, t.Q, fes.ne
        self.symm = True
        geom = _geometry(fes, t, modes)
        C, cdim = self._coefficient(fes, t, geom)
        self.B, self.G, self.W = to_dev(t.B), to_dev(t.G), to_dev(t.W)
        self.qdata = torch.empty(t.Q ** 3 * 6 * fes.ne, dtype=torch.float64, device=dev.torch_device)
        check(dev.lib.gbpa_diffusion_setup3d_nodes(dev.ctx, fes.ne, geom["dg"], t.Q, cdim, _p(self.W),
                                                   _p(geom["Bg"]), _p(geom["Gg"]), _p(geom["X"]),
                                                   _p(C), C.numel(), _p(self.qdata)),
              "diffusion_setup3d_nodes")

    def AddMultPA(self, x, y):
        dev = _dev()
        check(dev.lib.gbpa_diffusion_apply3d(dev.ctx, self.ne, 1, self.D, self.Q, _p(self.B), _p(self.G),
                                             None, None, _p(self.qdata), _p(x), _p(y)), "diffusion_apply3d")

    def AssembleDiagonalPA(self, y):
        dev = _dev()
        check(dev.lib.gbpa_diffusion_diagonal3d(dev.ctx, self.ne, 1, self.D, self.Q, _p(self.B),
                                                _p(self.G), _p(self.qdata), _p(y)), "diffusion_diagonal3d")


class MassIntegrator(_PAIntegrator):
    kind = _lib.GBPA_MASS

    def AssemblePA(self, fes, modes=None):
        dev = _dev()
        p = fes.p
        self.tables = t = Tables(p, self.quad_points(p))
        self.fes = fes
        self.D, self.Q, self.ne = t.D, t.Q, fes.ne
        self.symm = True
        geom = _geometry(fes, t, modes)
        C, _ = self._coefficient(fes, t, geom)
        self.B, self.G, self.W = to_dev(t.B), to_dev(t.G), to_dev(t.W)
        detJ = torch.empty(t.Q ** 3 * fes.ne, dtype=torch.float64, device=dev.torch_device)
        check(dev.lib.gbpa_geom_determinants3d(dev.ctx, fes.ne, geom["dg"], t.Q, _p(geom["Bg"]),
                                               _p(geom["Gg"]), _p(geom["X"]), _p(detJ)), "geom_det")
        self.qdata = torch.empty_like(detJ)
        check(dev.lib.gbpa_mass_setup3d(dev.ctx, fes.ne, t.Q ** 3, _p(self.W), _p(detJ), _p(C), C.numel(),
                                        1, _p(self.qdata)), "mass_setup3d")

    def AddMultPA(self, x, y):
        dev = _dev()
        check(dev.lib.gbpa_mass_apply3d(dev.ctx, self.ne, self.D, self.Q, _p(self.B), None,
                                        _p(self.qdata), _p(x), _p(y)), "mass_apply3d")

    def AssembleDiagonalPA(self, y):
        dev = _dev()
        check(dev.lib.gbpa_mass_diagonal3d(dev.ctx, self.ne, self.D, self.Q, _p(self.B),
                                           _p(self.qdata), _p(y)), "mass_diagonal3d")


class DomainLFIntegrator(_PAIntegrator):
    """fem/lininteg.hpp DomainLFIntegrator(f): b_i = (f, phi_i), assembled on
    the device. Default rule: order 2p (p + 1 Gauss points per direction)."""

    def quad_points(self, p):
        return self.ir_points if self.ir_points else p + 1


class LinearForm:
    """fem/linearform.cpp LinearForm with device assembly (UseFastAssembly,
    LinearFormExtension::Assemble): the sum of its domain integrators."""

    def __init__(self, fes):
        self.fes = fes
        self.integs = []
        self.b = None

    def AddDomainIntegrator(self, lfi):
        self.integs.append(lfi)

    def Assemble(self, modes=None):
        dev = _dev()
        fes = self.fes
        R = fes.GetElementRestriction()
        self.b = torch.zeros(fes.ndofs, dtype=torch.float64, device=dev.torch_device)
        part = torch.empty_like(self.b)
        for lfi in self.integs:
            t = Tables(fes.p, lfi.quad_points(fes.p))
            geom = _geometry(fes, t, modes)
            detJ = torch.empty(t.Q ** 3 * fes.ne, dtype=torch.float64, device=dev.torch_device)
            check(dev.lib.gbpa_geom_determinants3d(dev.ctx, fes.ne, geom["dg"], t.Q, _p(geom["Bg"]), _p(geom["Gg"]),
                                                   _p(geom["X"]), _p(detJ)), "geom_determinants3d")
            C, _ = lfi._coefficient(fes, t, geom)
            B, W = to_dev(t.B), to_dev(t.W)
            check(dev.lib.gbpa_domain_lf3d(dev.ctx, fes.ne, t.D, t.Q, _p(B), _p(W), _p(detJ), _p(C), C.numel(),
                                           fes.ndofs, _p(R.offsets), _p(R.indices), _p(part)), "domain_lf3d")
            self.b += part
        return self.b


class PAOperator:
    """The library's fused L-vector operator (restriction + integrator +
    transpose, optionally constrained): one gbpa_operator."""

    def __init__(self, kind, fes_or_maps, D, Q, B, G, qdata, ess=None, precision=_lib.GBPA_F64,
                 symm=True, scatter=_lib.GBPA_SCATTER_CSR):
        dev = _dev()
        R = fes_or_maps.GetElementRestriction() if hasattr(fes_or_maps, "GetElementRestriction") else fes_or_maps
        self.R = R
        # GBPA_F64X2 keeps FP64 data (the library splits qdata internally)
        dt = torch.float32 if precision == _lib.GBPA_F32 else torch.float64
        self.dtype = dt
        self.B, self.G, self.qdata = B.to(dt).contiguous(), G.to(dt).contiguous(), qdata.to(dt).contiguous()
        self.ess = to_dev(np.asarray(ess, np.int32)) if ess is not None and len(ess) else None
        self.ndofs = R.ndofs
        desc = _lib.OperatorDesc(kind, precision, R.ne, R.ndofs, D, Q, 1 if symm else 0,
                                 self.B.data_ptr(), self.G.data_ptr(), self.qdata.data_ptr(),
                                 R.gather_map.data_ptr(), R.offsets.data_ptr(), R.indices.data_ptr(),
                                 self.ess.data_ptr() if self.ess is not None else None,
                                 0 if self.ess is None else self.ess.numel(), scatter)
        h = ctypes.c_void_p()
        check(dev.lib.gbpa_operator_create(dev.ctx, ctypes.byref(desc), ctypes.byref(h)), "operator_create")
        self.handle = h

    def Height(self):
        return self.ndofs

    def Mult(self, x, y):
        check(_dev().lib.gbpa_operator_mult(self.handle, _p(x), _p(y)), "operator_mult")

    def MultHost(self, x, y):
        """Mult of host (CPU) tensors; returns when y holds the result. Pinned
        tensors are read and written by the kernels in place; pageable ones
        are staged through device scratch."""
        if x.device.type != "cpu" or y.device.type != "cpu":
            raise ValueError("MultHost takes CPU tensors")
        if not (x.is_contiguous() and y.is_contiguous()) or x.numel() != self.ndofs or y.numel() != self.ndofs:
            raise ValueError("MultHost takes contiguous vectors of ndofs entries")
        check(_dev().lib.gbpa_operator_mult_host(self.handle, _p(x), _p(y)), "operator_mult_host")

    def AssembleDiagonal(self, diag):
        check(_dev().lib.gbpa_operator_assemble_diagonal(self.handle, _p(diag)), "operator_assemble_diagonal")

    def SetElementMarkers(self, attributes, markers):
        """Only elements whose attribute a has markers[a - 1] != 0 contribute
        (AddMultWithMarkers, fem/bilinearform_ext.cpp:807-847); None removes
        the markers."""
        lib = _dev().lib
        if attributes is None:
            check(lib.gbpa_operator_set_element_markers(self.handle, None, None, 0), "set_element_markers")
            return
        a = to_dev(np.asarray(attributes, np.int32))
        m = to_dev(np.asarray(markers, np.int32))
        check(lib.gbpa_operator_set_element_markers(self.handle, _p(a), _p(m), m.numel()),
              "set_element_markers")

    def __del__(self):
        try:
            _dev().lib.gbpa_operator_destroy(self.handle)
        except Exception:
            pass


class BilinearForm:
    """BilinearForm with AssemblyLevel::PARTIAL and one domain integrator
    (fem/bilinearform.cpp, fem/bilinearform_ext.cpp)."""

    def __init__(self, fes):
        self.fes = fes
        self.integs = []
        self.level = AssemblyLevel.LEGACY
        self.op = None

    def SetAssemblyLevel(self, level):
        if level != AssemblyLevel.PARTIAL:
            raise NotImplementedError("only AssemblyLevel.PARTIAL is provided")
        self.level = level

    def AddDomainIntegrator(self, integ, elem_marker=None):
        """elem_marker: one entry per element attribute (the mesh's
        `attributes`); only elements of marked attributes contribute."""
        if self.integs:
            raise NotImplementedError("one domain integrator per form")
        self.integs.append(integ)
        self.elem_marker = None if elem_marker is None else np.asarray(elem_marker, np.int32)

    def _markers(self, op):
        if getattr(self, "elem_marker", None) is not None:
            op.SetElementMarkers(self.fes.mesh.attributes, self.elem_marker)
        return op

    def Assemble(self, modes=None, precision=_lib.GBPA_F64):
        if self.level != AssemblyLevel.PARTIAL:
            raise RuntimeError("call SetAssemblyLevel(AssemblyLevel.PARTIAL) first")
        integ = self.integs[0]
        integ.AssemblePA(self.fes, modes)
        self.op = self._markers(PAOperator(integ.kind, self.fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata,
                                           precision=precision))

    def Height(self):
        return self.fes.ndofs

    def Mult(self, x, y):
        self.op.Mult(x, y)

    def AssembleDiagonal(self, diag):
        self.op.AssembleDiagonal(diag)

    def ConstrainedOperator(self, ess, precision=_lib.GBPA_F64):
        integ = self.integs[0]
        return self._markers(PAOperator(integ.kind, self.fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata,
                                        ess=ess, precision=precision))

    def FormLinearSystem(self, ess_tdof_list, x, b):
        """Operator::FormLinearSystem (linalg/operator.cpp:129-143) with the
        ConstrainedOperator's EliminateRHS (linalg/operator.cpp:574-599):
        B = b - A x_ess, B[ess] = x[ess]; X = x."""
        A = self.ConstrainedOperator(ess_tdof_list)
        ess = A.ess
        w = torch.zeros_like(x)
        if ess is not None:
            w[ess.long()] = x[ess.long()]
        z = torch.empty_like(x)
        self.op.Mult(w, z)
        B = b - z
        if ess is not None:
            B[ess.long()] = x[ess.long()]
        return A, x.clone(), B


class OperatorJacobiSmoother:
    """linalg/solvers.cpp:331-452 (non-iterative mode, damping 1)."""

    def __init__(self, a, ess_tdof_list, damping=1.0):
        dev = _dev()
        n = a.Height()
        diag = torch.empty(n, dtype=torch.float64, device=dev.torch_device)
        a.AssembleDiagonal(diag)
        self.dinv = torch.empty_like(diag)
        ess = to_dev(np.asarray(ess_tdof_list, np.int32)) if len(ess_tdof_list) else None
        check(dev.lib.gbpa_jacobi_setup(dev.ctx, n, _p(diag), _p(ess), 0 if ess is None else ess.numel(),
                                        damping, _p(self.dinv)), "jacobi_setup")

    def Mult(self, x, y):
        y.copy_(self.dinv * x)


class CGSolver:
    """linalg/solvers.cpp:869-1050 on the device (see gbpa_pcg_solve)."""

    def __init__(self):
        self.rel_tol, self.abs_tol, self.max_iter = 0.0, 0.0, 10
        self.oper, self.prec, self.iterative_mode = None, None, False
        self.info = _lib.SolveInfo()

    def SetRelTol(self, t): self.rel_tol = t
    def SetAbsTol(self, t): self.abs_tol = t
    def SetMaxIter(self, m): self.max_iter = m
    def SetOperator(self, A): self.oper = A
    def SetPreconditioner(self, M): self.prec = M
    def SetPrintLevel(self, _): pass

    def Mult(self, b, x):
        if isinstance(self.prec, Multigrid):
            st = _dev().lib.gbpa_pcg_solve_mg(self.oper.handle, self.prec.handle, _p(b), _p(x), self.rel_tol,
                                              self.abs_tol, self.max_iter, ctypes.byref(self.info))
            if st not in (0, -6):
                check(st, "pcg_solve_mg")
            return
        if self.prec is None:
            dinv = torch.ones_like(b)
        else:
            dinv = self.prec.dinv
        st = _dev().lib.gbpa_pcg_solve(self.oper.handle, _p(dinv), _p(b), _p(x), self.rel_tol,
                                       self.abs_tol, self.max_iter, 1 if self.iterative_mode else 0,
                                       ctypes.byref(self.info))
        if st not in (0, -6):
            check(st, "pcg_solve")

    def GetNumIterations(self): return self.info.iterations
    def GetFinalNorm(self): return self.info.final_norm
    def GetConverged(self): return bool(self.info.converged)


# ------------------------------------------------------------ p-multigrid
class TransferOperator:
    """fem/transfer.cpp TransferOperator between two H1 spaces of different
    orders on the same mesh (TensorProductPRefinementTransferOperator):
    Mult prolongs lfes -> hfes, MultTranspose restricts."""

    def __init__(self, lfes, hfes, precision=_lib.GBPA_F64):
        dev = _dev()
        from . import fem
        Rl, Rh = lfes.GetElementRestriction(), hfes.GetElementRestriction()
        dc, df = lfes.p + 1, hfes.p + 1
        Bi, _ = fem.basis_tables(fem.gauss_lobatto(dc), fem.gauss_lobatto(df))
        self.Bi = np.ascontiguousarray(Bi, np.float64)
        self.lfes, self.hfes = lfes, hfes
        h = ctypes.c_void_p()
        check(dev.lib.gbpa_ptransfer_create(dev.ctx, lfes.ne, dc, lfes.ndofs, _p(Rl.gather_map), _p(Rl.offsets),
                                            _p(Rl.indices), df, hfes.ndofs, _p(Rh.gather_map), _p(Rh.offsets),
                                            _p(Rh.indices), self.Bi.ctypes.data_as(ctypes.c_void_p),
                                            _lib.GBPA_F32 if precision == _lib.GBPA_F32 else _lib.GBPA_F64,
                                            ctypes.byref(h)), "ptransfer_create")
        self.handle = h

    def Mult(self, x, y):
        check(_dev().lib.gbpa_ptransfer_mult(self.handle, _p(x), _p(y)), "ptransfer_mult")

    def MultTranspose(self, x, y):
        check(_dev().lib.gbpa_ptransfer_mult_transpose(self.handle, _p(x), _p(y)), "ptransfer_mult_transpose")

    def __del__(self):
        try:
            _dev().lib.gbpa_ptransfer_destroy(self.handle)
        except Exception:
            pass


class OperatorChebyshevSmoother:
    """linalg/solvers.cpp OperatorChebyshevSmoother on a constrained
    PAOperator. max_eig_estimate None: PowerMethod (power_iterations,
    power_tolerance) from a splitmix64 start vector of power_seed."""

    def __init__(self, oper, diag, ess_tdof_list, order, max_eig_estimate=None, power_iterations=10,
                 power_tolerance=1e-8, power_seed=12345):
        dev = _dev()
        self.oper, self.diag = oper, diag
        h = ctypes.c_void_p()
        lam = float(max_eig_estimate) if max_eig_estimate else 0.0
        check(dev.lib.gbpa_chebyshev_create(oper.handle, _p(diag), order, lam, power_iterations, power_tolerance,
                                            power_seed, ctypes.byref(h)), "chebyshev_create")
        self.handle = h

    def GetMaxEigEstimate(self):
        v = ctypes.c_double(0.0)
        check(_dev().lib.gbpa_chebyshev_get_max_eig(self.handle, ctypes.byref(v)), "chebyshev_get_max_eig")
        return v.value

    def Mult(self, x, y):
        check(_dev().lib.gbpa_chebyshev_mult(self.handle, _p(x), _p(y)), "chebyshev_mult")

    def __del__(self):
        try:
            _dev().lib.gbpa_chebyshev_destroy(self.handle)
        except Exception:
            pass


class Multigrid:
    """fem/multigrid.cpp Multigrid with a V(1,1) cycle: operators coarsest
    first, Chebyshev smoothers on levels >= 1, prolongations between
    consecutive levels; level 0 solved by CG to coarse_rel_tol."""

    def __init__(self, operators, smoothers, prolongations, coarse_rel_tol=1e-2, coarse_max_it=200,
                 coarse_jacobi=False, coarse_diag=None):
        dev = _dev()
        nl = len(operators)
        self.operators, self.smoothers, self.prolongations = operators, smoothers, prolongations
        ops = (ctypes.c_void_p * nl)(*[o.handle for o in operators])
        sms = (ctypes.c_void_p * nl)(*[None] + [s.handle for s in smoothers[1:]])
        prs = (ctypes.c_void_p * max(nl - 1, 1))(*[P.handle for P in prolongations])
        h = ctypes.c_void_p()
        check(dev.lib.gbpa_multigrid_create(dev.ctx, nl, ops, sms, prs, coarse_rel_tol, coarse_max_it,
                                            1 if coarse_jacobi else 0, _p(coarse_diag), ctypes.byref(h)),
              "multigrid_create")
        self.handle = h

    def Mult(self, x, y):
        check(_dev().lib.gbpa_multigrid_mult(self.handle, _p(x), _p(y)), "multigrid_mult")

    def __del__(self):
        try:
            _dev().lib.gbpa_multigrid_destroy(self.handle)
        except Exception:
            pass


class DiffusionMultigrid(Multigrid):
    """The reference's examples/ex26.cpp DiffusionMultigrid on one mesh with
    an order hierarchy (e.g. 1, 2, 4): a constrained PA diffusion operator
    per order (Dirichlet on the whole boundary), order-2 Chebyshev smoothers
    with power-method eigenvalue estimates, CG to 1e-2 on the coarsest
    order (coarse_jacobi: Jacobi-preconditioned). precision: the levels'
    arithmetic (GBPA_F64, GBPA_F64X2, or GBPA_F32 for an FP32 V-cycle that
    preconditions the FP64 CG). max_eigs: optional eigenvalue estimates for
    levels 1.. (else estimated)."""

    def __init__(self, mesh, orders, coeff="kappa", modes=None, precision=_lib.GBPA_F64, cheb_order=2,
                 coarse_rel_tol=1e-2, coarse_max_it=200, max_eigs=None, ir_points=None, coarse_jacobi=False):
        dev = _dev()
        self.spaces, self.integs, ops, smoothers, prols = [], [], [], [], []
        self.ess = []
        coarse_diag = None
        for l, p in enumerate(orders):
            fes = FiniteElementSpace(mesh, p)
            integ = DiffusionIntegrator(coeff, ir_points=ir_points(p) if ir_points else None)
            integ.AssemblePA(fes, modes=modes)
            ess = fes.GetBoundaryTrueDofs()
            A = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=ess, precision=precision)
            self.spaces.append(fes); self.integs.append(integ); self.ess.append(ess)
            ops.append(A)
            # the diagonal comes from the FP64 data (an FP32 operator cannot assemble it)
            A64 = A if precision != _lib.GBPA_F32 else PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G,
                                                                   integ.qdata, ess=ess)
            diag = torch.empty(fes.ndofs, dtype=torch.float64, device=dev.torch_device)
            A64.AssembleDiagonal(diag)
            del A64
            if l == 0:
                smoothers.append(None)
                coarse_diag = diag
            else:
                lam = max_eigs[l - 1] if max_eigs is not None else None
                smoothers.append(OperatorChebyshevSmoother(A, diag, ess, cheb_order, lam))
                prols.append(TransferOperator(self.spaces[l - 1], fes, precision))
        self.coarse_diag = coarse_diag
        super().__init__(ops, smoothers, prols, coarse_rel_tol, coarse_max_it, coarse_jacobi,
                         coarse_diag if coarse_jacobi else None)
