"""ctypes bindings of the C oracle ``liboracle.so`` (TEST INFRASTRUCTURE ONLY).

Thin numpy wrappers around oracle/pf2_oracle.c; every array is passed as a
contiguous float64 / int32 buffer.  The library is built by ``make -C oracle``
(``__graft_entry__.build()`` does it).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

D = np.float64
I = np.int32
_dp = np.ctypeslib.ndpointer(dtype=D, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=I, flags="C_CONTIGUOUS")


class Params(C.Structure):
    _fields_ = [("rho", C.c_double), ("mu", C.c_double), ("dt", C.c_double), ("tol", C.c_double),
                ("maxit", C.c_int), ("scheme", C.c_int), ("substeps", C.c_int), ("level", C.c_int),
                ("n_outer", C.c_int), ("pressure_precond", C.c_int),
                ("calc_loads", C.c_int), ("body_id", C.c_int),
                ("thickness", C.c_double), ("mean_velocity", C.c_double),
                ("lx", C.c_double), ("ly", C.c_double),
                ("has_cylinder", C.c_int),
                ("cx", C.c_double), ("cy", C.c_double), ("radius", C.c_double),
                ("pressure_ordering", C.c_int), ("prediction_solver", C.c_int), ("gmres_orth", C.c_int),
                ("pressure_criterion", C.c_int), ("pressure_tol", C.c_double), ("pressure_maxit", C.c_int)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("residual", C.c_double)]


class StepInfo(C.Structure):
    _fields_ = [("particles", C.c_int), ("deleted", C.c_int), ("added", C.c_int),
                ("it_pred", (C.c_int * 8) * 2), ("it_pres", C.c_int * 8), ("it_corr", (C.c_int * 8) * 2),
                ("conv_ok", C.c_int), ("cx", C.c_double), ("cy", C.c_double), ("res_pres", C.c_double * 8)]


PRECOND = {"none": -1, "jacobi": 0, "ilu": 1, "ic": 2}


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            subprocess.run(["make", "-C", _HERE], check=True, capture_output=True)
        _lib = C.CDLL(_LIB)
        _declare(_lib)
    return _lib


def _declare(L):
    vp = C.c_void_p
    L.or_mesh_geometry.argtypes = [C.c_int, _dp, _ip, _dp, _dp]
    L.or_node_cells.argtypes = [C.c_int, C.c_int, _ip, _ip, vp]
    L.or_node_cells.restype = C.c_int
    L.or_neighbors.argtypes = [C.c_int, C.c_int, _ip, _ip, vp]
    L.or_neighbors.restype = C.c_int
    L.or_csr_structure.argtypes = [C.c_int, C.c_int, _ip, _ip, vp]
    L.or_csr_structure.restype = C.c_int
    L.or_edge_boundary_ids.argtypes = [C.c_int, _dp, _ip, C.c_double, C.c_double, C.c_int,
                                       C.c_double, C.c_double, C.c_double, _ip]
    L.or_spmv.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _dp]
    L.or_assemble_poisson.argtypes = [C.c_int, _dp, _ip, _dp, _dp, C.c_int, C.c_double, _ip, _ip, _dp, _dp]
    L.or_apply_bcs.argtypes = [C.c_int, _ip, _ip, _dp, _dp, C.c_int, _ip, _dp]
    L.or_ilu0.argtypes = [C.c_int, _ip, _ip, _dp]
    L.or_ic0.argtypes = [C.c_int, _ip, _ip, _dp]
    for fn in (L.or_pcg, L.or_gmres):
        fn.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _dp, C.c_double, C.c_int, C.c_int, C.POINTER(SolveInfo)]
        fn.restype = C.c_int
    L.or_subcell_centers.argtypes = [C.c_int, _dp]
    L.or_subcell_centers.restype = C.c_int
    L.or_determine_subcell.argtypes = [C.c_int, C.c_double, _dp]
    L.or_determine_subcell.restype = C.c_int
    L.or_seed.argtypes = [C.c_int, _dp, _ip, C.c_int, _dp] + [_dp] * 7 + [_ip]
    L.or_seed.restype = C.c_int
    L.or_correct_velocity.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _dp, _dp, _dp, vp, vp, _dp, _dp]
    L.or_project.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _dp, _dp, _dp, C.c_int, _dp, _dp]
    L.or_advect.argtypes = ([C.c_int, C.c_int] + [_dp] * 7 + [_ip, C.c_int, _dp, C.c_int, _ip, _dp, _ip, _ip,
                            _dp, _dp, C.c_double, C.c_int, C.c_int, _dp, C.POINTER(C.c_int), C.POINTER(C.c_int)])
    L.or_advect.restype = C.c_int
    L.or_locate.argtypes = [C.c_double, C.c_double, C.c_int, _dp, _ip, _dp, _ip, _ip, _dp]
    L.or_locate.restype = C.c_int
    L.or_assemble_prediction.argtypes = ([C.c_int, _dp, _ip, _dp, _dp, _ip, C.POINTER(Params)] + [_dp] * 4 +
                                         [vp, _ip, _ip, _dp, _dp, _dp, _dp])
    L.or_assemble_pressure.argtypes = [C.c_int, _ip, _dp, _dp, C.POINTER(Params), _dp, _dp, vp, _ip, _ip, _dp, _dp]
    L.or_assemble_correction.argtypes = ([C.c_int, _ip, _dp, _dp, C.POINTER(Params), _dp, _dp, _dp, vp, _ip, _ip]
                                         + [_dp] * 4)
    L.or_prediction_bc.argtypes = [C.c_int, _ip, _dp, _dp, C.POINTER(Params), _dp, vp, C.c_int, _ip, _dp, _ip,
                                   C.c_int, _dp]
    L.or_body_loads.argtypes = [C.c_int, _dp, _ip, _dp, _ip, C.POINTER(Params), _dp, _dp, _dp, _dp]
    L.or_body_loads.restype = C.c_int
    L.or_flow_create.argtypes = ([C.c_int, _dp, C.c_int, _ip, C.POINTER(Params)] +
                                 [C.c_int, _ip, _dp] * 3 + [C.c_int])
    L.or_flow_create.restype = vp
    L.or_flow_destroy.argtypes = [vp]
    L.or_flow_step.argtypes = [vp, C.POINTER(StepInfo)]
    L.or_flow_step.restype = C.c_int
    L.or_flow_particle_count.argtypes = [vp]
    L.or_flow_particle_count.restype = C.c_int
    L.or_flow_get_field.argtypes = [vp, C.c_int, _dp]
    L.or_flow_set_field.argtypes = [vp, C.c_int, _dp]
    L.or_flow_get_particles.argtypes = [vp] + [_dp] * 7 + [_ip]
    L.or_flow_set_particles.argtypes = [vp, C.c_int] + [_dp] * 7 + [_ip]
    L.or_flow_csr_nnz.argtypes = [vp]
    L.or_flow_csr_nnz.restype = C.c_int
    L.or_flow_get_matrix.argtypes = [vp, C.c_int, _dp, _dp]
    L.or_multicolour_order.argtypes = [C.c_int, _ip, _ip, C.c_int, _ip, vp]
    L.or_multicolour_order.restype = C.c_int
    L.or_cg.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _dp, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                        C.POINTER(SolveInfo), C.POINTER(C.c_double)]
    L.or_cg.restype = C.c_int
    L.or_bicgstab.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _dp, C.c_double, C.c_int, C.c_int, C.c_int,
                              C.POINTER(SolveInfo)]
    L.or_bicgstab.restype = C.c_int
    L.or_gmres_cgs2.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _dp, C.c_double, C.c_int, C.c_int,
                                C.POINTER(SolveInfo)]
    L.or_gmres_cgs2.restype = C.c_int
    L.or_flow_set_solvers.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
    L.or_mesh3d_geometry.argtypes = [C.c_int, _dp, _ip, _dp, _dp]
    L.or_mesh3d_neighbors.argtypes = [C.c_int, _ip, _ip, vp]
    L.or_mesh3d_neighbors.restype = C.c_int
    L.or_csr_structure_3d.argtypes = [C.c_int, C.c_int, _ip, _ip, vp]
    L.or_csr_structure_3d.restype = C.c_int
    L.or_cell_quadrature_3d.argtypes = [_dp, _dp]
    L.or_cell_quadrature_3d.restype = C.c_int
    L.or_assemble_poisson_3d.argtypes = [C.c_int, _dp, _ip, _dp, _dp, C.c_int, C.c_double, _ip, _ip, _dp, _dp]


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# ---- mesh -------------------------------------------------------------------
def mesh_geometry(xy, tri):
    xy, tri = _c(xy, D), _c(tri, I)
    nc = tri.shape[0]
    area = np.empty(nc, D)
    invJ = np.empty((nc, 4), D)
    lib().or_mesh_geometry(nc, xy, tri, area, invJ)
    return area, invJ


def neighbors(nv, tri):
    tri = _c(tri, I)
    nc = tri.shape[0]
    off = np.empty(nc + 1, I)
    n = lib().or_neighbors(nv, nc, tri, off, None)
    idx = np.empty(max(n, 1), I)
    lib().or_neighbors(nv, nc, tri, off, _ptr(idx))
    return off, idx[:n]


def csr_structure(nv, tri):
    tri = _c(tri, I)
    nc = tri.shape[0]
    rp = np.empty(nv + 1, I)
    n = lib().or_csr_structure(nv, nc, tri, rp, None)
    col = np.empty(max(n, 1), I)
    lib().or_csr_structure(nv, nc, tri, rp, _ptr(col))
    return rp, col[:n]


def node_cells(nv, tri):
    tri = _c(tri, I)
    off = np.empty(nv + 1, I)
    n = lib().or_node_cells(nv, tri.shape[0], tri, off, None)
    cells = np.empty(max(n, 1), I)
    lib().or_node_cells(nv, tri.shape[0], tri, off, _ptr(cells))
    return off, cells[:n]


# ---- 3D mesh and Poisson3D ----------------------------------------------------
def mesh3d_geometry(xyz, tet):
    xyz, tet = _c(xyz, D), _c(tet, I)
    nc = tet.shape[0]
    vol = np.empty(nc, D)
    invJ = np.empty((nc, 3, 3), D)
    lib().or_mesh3d_geometry(nc, xyz, tet, vol, invJ)
    return vol, invJ


def mesh3d_neighbors(tet):
    tet = _c(tet, I)
    nc = tet.shape[0]
    off = np.empty(nc + 1, I)
    n = lib().or_mesh3d_neighbors(nc, tet, off, None)
    idx = np.empty(max(n, 1), I)
    lib().or_mesh3d_neighbors(nc, tet, off, _ptr(idx))
    return off, idx[:n]


def csr_structure_3d(nv, tet):
    tet = _c(tet, I)
    nc = tet.shape[0]
    rp = np.empty(nv + 1, I)
    n = lib().or_csr_structure_3d(nv, nc, tet, rp, None)
    col = np.empty(max(n, 1), I)
    lib().or_csr_structure_3d(nv, nc, tet, rp, _ptr(col))
    return rp, col[:n]


def cell_quadrature_3d():
    c, w = np.empty(24, D), np.empty(6, D)
    n = lib().or_cell_quadrature_3d(c, w)
    return c.reshape(-1, 4)[:n], w[:n]


def assemble_poisson_3d(xyz, tet, vol, invJ, rowptr, col, rhs_kind=0, lam=0.5):
    val = np.zeros(col.size, D)
    rhs = np.zeros(xyz.shape[0], D)
    lib().or_assemble_poisson_3d(tet.shape[0], _c(xyz, D), _c(tet, I), _c(vol, D), _c(invJ, D), rhs_kind, lam,
                                 _c(rowptr, I), _c(col, I), val, rhs)
    return val, rhs


def edge_boundary_ids(xy, tri, lx, ly, cylinder=None):
    xy, tri = _c(xy, D), _c(tri, I)
    ids = np.empty((tri.shape[0], 3), I)
    cx, cy, r = cylinder if cylinder is not None else (0.0, 0.0, 0.0)
    lib().or_edge_boundary_ids(tri.shape[0], xy, tri, lx, ly, int(cylinder is not None), cx, cy, r, ids)
    return ids


# ---- assembly / BCs / solvers -------------------------------------------------
def assemble_poisson(xy, tri, area, invJ, rowptr, col, rhs_kind=1, lam=1.0):
    val = np.zeros(col.size, D)
    rhs = np.zeros(xy.shape[0], D)
    lib().or_assemble_poisson(tri.shape[0], _c(xy, D), _c(tri, I), _c(area, D), _c(invJ, D),
                              rhs_kind, lam, _c(rowptr, I), _c(col, I), val, rhs)
    return val, rhs


def apply_bcs(rowptr, col, val, rhs, bc_nodes, bc_vals):
    val, rhs = val.copy(), rhs.copy()
    lib().or_apply_bcs(rowptr.size - 1, _c(rowptr, I), _c(col, I), val, rhs, len(bc_nodes),
                       _c(bc_nodes, I), _c(bc_vals, D))
    return val, rhs


def spmv(rowptr, col, val, x):
    y = np.empty(rowptr.size - 1, D)
    lib().or_spmv(rowptr.size - 1, _c(rowptr, I), _c(col, I), _c(val, D), _c(x, D), y)
    return y


def pcg(rowptr, col, val, b, x0=None, tol=1e-8, maxit=1000, precond="jacobi"):
    n = rowptr.size - 1
    x = np.zeros(n, D) if x0 is None else _c(x0, D).copy()
    info = SolveInfo()
    lib().or_pcg(n, _c(rowptr, I), _c(col, I), _c(val, D), x, _c(b, D), tol, maxit, PRECOND[precond], C.byref(info))
    return x, info


def gmres(rowptr, col, val, b, x0=None, tol=1e-8, maxit=1000, precond="jacobi"):
    n = rowptr.size - 1
    x = np.zeros(n, D) if x0 is None else _c(x0, D).copy()
    info = SolveInfo()
    lib().or_gmres(n, _c(rowptr, I), _c(col, I), _c(val, D), x, _c(b, D), tol, maxit, PRECOND[precond],
                   C.byref(info))
    return x, info


def multicolour_order(rowptr, col, kempe=True):
    """(perm, colour starts): the multicolour order of the engine's ILU(0)/IC(0) option."""
    n = rowptr.size - 1
    perm = np.empty(n, I)
    starts = np.empty(n + 2, I)
    nc = lib().or_multicolour_order(n, _c(rowptr, I), _c(col, I), int(kempe), perm, starts.ctypes.data_as(C.c_void_p))
    return perm, starts[:nc + 1].copy()


def cg(rowptr, col, val, b, x0=None, tol=1e-8, maxit=1000, precond="jacobi", ordering=0, criterion=0):
    """CG with the engine's options: ordering 1 = multicolour ILU/IC, criterion 1 = relative.
    Returns (x, info, final ||r|| / ||b||)."""
    n = rowptr.size - 1
    x = np.zeros(n, D) if x0 is None else _c(x0, D).copy()
    info = SolveInfo()
    rel = C.c_double()
    lib().or_cg(n, _c(rowptr, I), _c(col, I), _c(val, D), x, _c(b, D), tol, maxit, PRECOND[precond], ordering,
                criterion, C.byref(info), C.byref(rel))
    return x, info, rel.value


def bicgstab(rowptr, col, val, b, x0=None, tol=1e-8, maxit=1000, precond="jacobi", criterion=0):
    n = rowptr.size - 1
    x = np.zeros(n, D) if x0 is None else _c(x0, D).copy()
    info = SolveInfo()
    lib().or_bicgstab(n, _c(rowptr, I), _c(col, I), _c(val, D), x, _c(b, D), tol, maxit, PRECOND[precond],
                      criterion, C.byref(info))
    return x, info


def gmres_cgs2(rowptr, col, val, b, x0=None, tol=1e-8, maxit=1000, precond="jacobi"):
    n = rowptr.size - 1
    x = np.zeros(n, D) if x0 is None else _c(x0, D).copy()
    info = SolveInfo()
    lib().or_gmres_cgs2(n, _c(rowptr, I), _c(col, I), _c(val, D), x, _c(b, D), tol, maxit, PRECOND[precond],
                        C.byref(info))
    return x, info


def ilu0(rowptr, col, val):
    f = _c(val, D).copy()
    lib().or_ilu0(rowptr.size - 1, _c(rowptr, I), _c(col, I), f)
    return f


def ic0(rowptr, col, val):
    f = _c(val, D).copy()
    lib().or_ic0(rowptr.size - 1, _c(rowptr, I), _c(col, I), f)
    return f


# ---- particles ------------------------------------------------------------------
def subcell_centers(level):
    c = np.zeros((16, 3), D)
    n = lib().or_subcell_centers(level, c)
    return c[: n * n]


def seed(xy, tri, level):
    nc = tri.shape[0]
    c3 = np.zeros((16, 3), D)
    lev = lib().or_subcell_centers(level, c3)
    np_ = nc * lev * lev
    arrs = [np.empty(np_, D) for _ in range(7)]
    cell = np.empty(np_, I)
    lib().or_seed(nc, _c(xy, D), _c(tri, I), lev, c3, *arrs, cell)
    return dict(x=arrs[0], y=arrs[1], l0=arrs[2], l1=arrs[3], l2=arrs[4], u=arrs[5], v=arrs[6], cell=cell)


def advect(P, xy, tri, invJ, nb_off, nb_idx, ux, uy, dt, substeps, level, cap=None):
    """Returns (particles dict, n_deleted, n_added)."""
    n = P["cell"].size
    cap = cap or max(2 * n, 16)
    arr = {k: np.zeros(cap, D) for k in ("x", "y", "l0", "l1", "l2", "u", "v")}
    cell = np.zeros(cap, I)
    for k in arr:
        arr[k][:n] = P[k]
    cell[:n] = P["cell"]
    c3 = np.zeros((16, 3), D)
    lev = lib().or_subcell_centers(level, c3)
    nd, na = C.c_int(0), C.c_int(0)
    m = lib().or_advect(n, cap, arr["x"], arr["y"], arr["l0"], arr["l1"], arr["l2"], arr["u"], arr["v"], cell,
                        xy.shape[0], _c(xy, D), tri.shape[0], _c(tri, I), _c(invJ, D), _c(nb_off, I),
                        _c(nb_idx, I), _c(ux, D), _c(uy, D), dt, substeps, lev, c3, C.byref(nd), C.byref(na))
    if m < 0:
        raise RuntimeError("oracle particle capacity exceeded")
    out = {k: v[:m].copy() for k, v in arr.items()}
    out["cell"] = cell[:m].copy()
    return out, nd.value, na.value


def project(P, tri, nv):
    ux, uy = np.empty(nv, D), np.empty(nv, D)
    lib().or_project(P["cell"].size, _c(tri, I), _c(P["cell"], I), _c(P["l0"], D), _c(P["l1"], D), _c(P["l2"], D),
                     _c(P["u"], D), _c(P["v"], D), nv, ux, uy)
    return ux, uy


def correct_velocity(P, tri, ux, uy, ux_old=None, uy_old=None):
    u, v = _c(P["u"], D).copy(), _c(P["v"], D).copy()
    uxo = None if ux_old is None else _c(ux_old, D)
    uyo = None if uy_old is None else _c(uy_old, D)
    lib().or_correct_velocity(P["cell"].size, _c(tri, I), _c(P["cell"], I), _c(P["l0"], D), _c(P["l1"], D),
                              _c(P["l2"], D), _c(ux, D), _c(uy, D), _ptr(uxo), _ptr(uyo), u, v)
    return u, v


def determine_subcell(level, l3):
    return lib().or_determine_subcell(level, 1.0 / level, _c(l3, D))


# ---- flow -----------------------------------------------------------------------
def make_params(**kw):
    p = Params()
    defaults = dict(rho=1.0, mu=1.0, dt=0.01, tol=1e-8, maxit=1000, scheme=0, substeps=3, level=2, n_outer=2,
                    pressure_precond=0, calc_loads=0, body_id=-1, thickness=1.0, mean_velocity=1.0,
                    lx=1.0, ly=1.0, has_cylinder=0, cx=0.2, cy=0.2, radius=0.05, pressure_ordering=0,
                    prediction_solver=1, gmres_orth=0, pressure_criterion=0, pressure_tol=0.0, pressure_maxit=0)
    defaults.update(kw)
    for k, v in defaults.items():
        setattr(p, k, v)
    return p


class Flow:
    """The oracle's full PFEM-2 step (Cylinder2D/main.cu:793-880) on host arrays."""

    FIELDS = {"ux": 0, "uy": 1, "ux_old": 2, "uy_old": 3, "pred_x": 4, "pred_y": 5, "p": 6, "p_old": 7}

    def __init__(self, xy, tri, params, bc_u, bc_v, bc_p, particle_cap=0):
        self.xy, self.tri = _c(xy, D), _c(tri, I)
        self.params = params
        self.nv = self.xy.shape[0]

        def split(b):
            n = np.array([i for i, _ in b], I) if b else np.zeros(1, I)
            v = np.array([g for _, g in b], D) if b else np.zeros(1, D)
            return len(b), n, v

        bu, bv, bp = split(bc_u), split(bc_v), split(bc_p)
        self._keep = (bu, bv, bp)
        self.h = lib().or_flow_create(self.nv, self.xy, self.tri.shape[0], self.tri, C.byref(params),
                                      *bu, *bv, *bp, particle_cap)

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_flow_destroy(self.h)
            self.h = None

    def step(self):
        info = StepInfo()
        rc = lib().or_flow_step(self.h, C.byref(info))
        if rc != 0:
            raise RuntimeError("oracle step failed (particle capacity)")
        return info

    def set_solvers(self, pressure_precond, pressure_ordering=0, prediction_solver=1, gmres_orth=0,
                    pressure_criterion=0):
        """The solver choices of the following steps; the state is kept."""
        lib().or_flow_set_solvers(self.h, pressure_precond, pressure_ordering, prediction_solver, gmres_orth,
                                  pressure_criterion)

    def field(self, name):
        out = np.empty(self.nv, D)
        lib().or_flow_get_field(self.h, self.FIELDS[name], out)
        return out

    def set_field(self, name, arr):
        lib().or_flow_set_field(self.h, self.FIELDS[name], _c(arr, D))

    def particles(self):
        n = lib().or_flow_particle_count(self.h)
        a = [np.empty(n, D) for _ in range(7)]
        cell = np.empty(n, I)
        lib().or_flow_get_particles(self.h, *a, cell)
        return dict(x=a[0], y=a[1], l0=a[2], l1=a[3], l2=a[4], u=a[5], v=a[6], cell=cell)

    def set_particles(self, P):
        n = P["cell"].size
        lib().or_flow_set_particles(self.h, n, *[_c(P[k], D) for k in ("x", "y", "l0", "l1", "l2", "u", "v")],
                                    _c(P["cell"], I))

    def matrix(self, which):
        nnz = lib().or_flow_csr_nnz(self.h)
        val, rhs = np.empty(nnz, D), np.empty(self.nv, D)
        lib().or_flow_get_matrix(self.h, which, val, rhs)
        return val, rhs


# ---- learned initial guess (message-passing network) -----------------------------
MPNN_H, MPNN_IN, MPNN_LAYERS = 64, 5, 3


def _declare_mpnn(L):
    L.or_mpnn_param_count.restype = C.c_int
    L.or_mpnn_forward.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _dp, C.c_void_p]
    L.or_mpnn_forward.restype = C.c_double
    L.or_mpnn_backward.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _dp, _dp]
    L.or_mpnn_backward.restype = C.c_double
    L.or_adamw.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                           C.c_double]


def mpnn_param_count():
    _declare_mpnn(lib())
    return lib().or_mpnn_param_count()


def mpnn_forward(rowptr, col, feat, theta, t=None):
    _declare_mpnn(lib())
    n = rowptr.size - 1
    y = np.empty(n, D)
    tt = None if t is None else _c(t, D)
    loss = lib().or_mpnn_forward(n, _c(rowptr, I), _c(col, I), _c(feat, D), _c(theta, D), y,
                                 None if tt is None else tt.ctypes.data_as(C.c_void_p))
    return y, loss


def mpnn_backward(rowptr, col, feat, theta, t):
    _declare_mpnn(lib())
    g = np.empty(mpnn_param_count(), D)
    loss = lib().or_mpnn_backward(rowptr.size - 1, _c(rowptr, I), _c(col, I), _c(feat, D), _c(theta, D), _c(t, D), g)
    return g, loss


def adamw(theta, grad, m, v, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8, wd=0.01):
    _declare_mpnn(lib())
    lib().or_adamw(theta.size, theta, _c(grad, D), m, v, step, lr, b1, b2, eps, wd)
