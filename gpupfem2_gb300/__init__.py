"""GB300-native PFEM-2 time-step engine (Python side of the C ABI in include/pf2.h).

The compute path is the CUDA library ``_build/libpf2.so`` (built by
``gpupfem2_gb300.build``); this module only binds it with ctypes and uses torch
tensors as device buffers and torch's current stream.  There is no CPU fallback:
loading fails loudly when the library is missing.

Classes mirror the reference's C++ API (andreyypopov/gpuPfem2): :class:`Mesh2D`,
:class:`SparseMatrixCSR`, :class:`DirichletBCs`, :class:`LinearSolver` (CG / GMRES
with Jacobi, ILU(0), IC(0)), :class:`ParticleHandler2D` and :class:`FlowEngine` (one
PFEM-2 time step of the channel drivers).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libpf2.so")
_lib = None

OK, NOT_CONVERGED, BAD_INPUT, OVERFLOW, CUDA_ERROR, TIMEOUT, IO_ERROR = range(7)
SOLVER_CG, SOLVER_GMRES, SOLVER_BICGSTAB = 0, 1, 2
PRECOND = {"none": -1, "jacobi": 0, "ilu": 1, "ic": 2}
CRITERION_ABS, CRITERION_REL = 0, 1
PRECISION_FP64, PRECISION_MIXED = 0, 1
X0_GIVEN, X0_LEARNED = 0, 1  # pf2_params.pressure_x0
RHS_GAUSSIAN, RHS_SINSIN = 0, 1
RHS3D_GAUSSIAN, RHS3D_SINSINSIN = 0, 1
CG_STANDARD, CG_ONE_REDUCTION, CG_PIPELINED = 0, 1, 2
FIELDS = {"ux": 0, "uy": 1, "ux_old": 2, "uy_old": 3, "pred_x": 4, "pred_y": 5, "p": 6, "p_old": 7}
MESH_FIELDS = {"xy": 0, "tri": 1, "area": 2, "inv_jacobi": 3, "neighbor_offsets": 4, "neighbor_indices": 5,
               "edge_ids": 6}


class Pf2Error(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (status %d)" % (msg, status))
        self.status = status


class Params(C.Structure):
    """pf2_params (SimulationParameters, src/parameters.cuh:6-51)."""
    _fields_ = [("rho", C.c_double), ("mu", C.c_double), ("dt", C.c_double), ("tolerance", C.c_double),
                ("max_iterations", C.c_int), ("scheme", C.c_int), ("substeps", C.c_int), ("level", C.c_int),
                ("n_outer", C.c_int), ("pressure_precond", C.c_int),
                ("calculate_loads", C.c_int), ("body_boundary_id", C.c_int),
                ("thickness", C.c_double), ("mean_velocity", C.c_double),
                ("body_cx", C.c_double), ("body_cy", C.c_double),
                ("pressure_precision", C.c_int), ("pressure_x0", C.c_int), ("gmres_restart", C.c_int),
                ("pressure_criterion", C.c_int), ("learn_steps", C.c_int), ("learn_rate", C.c_float),
                ("pressure_ordering", C.c_int), ("gmres_orthogonalization", C.c_int), ("cg_variant", C.c_int),
                ("prediction_solver", C.c_int), ("pressure_tolerance", C.c_double),
                ("pressure_max_iterations", C.c_int)]


class MeshView(C.Structure):
    _fields_ = [("nv", C.c_int), ("nc", C.c_int), ("n_neighbor_entries", C.c_int),
                ("xy", C.c_void_p), ("tri", C.c_void_p), ("area", C.c_void_p), ("inv_jacobi", C.c_void_p),
                ("neighbor_offsets", C.c_void_p), ("neighbor_indices", C.c_void_p),
                ("edge_boundary_ids", C.c_void_p)]


class DirichletNode(C.Structure):
    _fields_ = [("node", C.c_uint), ("value", C.c_double)]


class SolverOptions(C.Structure):
    _fields_ = [("kind", C.c_int), ("precond", C.c_int), ("tolerance", C.c_double), ("max_iterations", C.c_int),
                ("criterion", C.c_int), ("precision", C.c_int), ("restart", C.c_int), ("ordering", C.c_int),
                ("orthogonalization", C.c_int), ("cg_variant", C.c_int)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("residual", C.c_double),
                ("outer_iterations", C.c_int), ("status", C.c_int)]


class StepInfo(C.Structure):
    _fields_ = [("particles", C.c_int), ("it_prediction", (C.c_int * 8) * 2), ("it_pressure", C.c_int * 8),
                ("it_correction", (C.c_int * 8) * 2), ("converged", C.c_int), ("status", C.c_int),
                ("cx", C.c_double), ("cy", C.c_double), ("guess_used", C.c_int),
                ("guess_residual", C.c_double * 2), ("pressure_residual", C.c_double * 8)]


def lib():
    """The loaded C ABI library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise Pf2Error(CUDA_ERROR, "libpf2.so is not built (run gpupfem2_gb300.build.build())")
        _lib = C.CDLL(LIB_PATH)
        _lib.pf2_last_error.restype = C.c_char_p
        _lib.pf2_status_string.restype = C.c_char_p
    return _lib


def _check(status, what=""):
    if status != OK:
        raise Pf2Error(status, "%s: %s" % (what, lib().pf2_last_error().decode()))


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dev(t):
    return C.c_void_p(0 if t is None else t.data_ptr())


def default_params(**kw) -> Params:
    p = Params()
    _check(lib().pf2_params_default(C.byref(p)), "pf2_params_default")
    for k, v in kw.items():
        if k == "pressure_precond" and isinstance(v, str):
            v = PRECOND[v]
        setattr(p, k, v)
    return p


class Mesh2D:
    """Mesh2D (src/mesh_2d.cuh): vertices, triangles, areas, inverse Jacobians,
    vertex-sharing neighbour lists and the CSR pattern, built on the device."""

    def __init__(self, handle):
        self.h = handle
        nv, nc, nn = C.c_int(), C.c_int(), C.c_int()
        _check(lib().pf2_mesh_sizes(self.h, C.byref(nv), C.byref(nc), C.byref(nn)), "pf2_mesh_sizes")
        self.nv, self.nc, self.n_neighbor_entries = nv.value, nc.value, nn.value

    @classmethod
    def from_arrays(cls, xy, tri, fill_neighbors=True):
        xy = np.ascontiguousarray(xy, dtype=np.float64)
        tri = np.ascontiguousarray(tri, dtype=np.int32)
        h = C.c_void_p()
        _check(lib().pf2_mesh_create(int(xy.shape[0]), xy.ctypes.data_as(C.c_void_p), int(tri.shape[0]),
                                     tri.ctypes.data_as(C.c_void_p), int(fill_neighbors), None, C.byref(h)),
               "pf2_mesh_create")
        return cls(h)

    @classmethod
    def load_dat(cls, path, fill_neighbors=True, scale=1.0):
        h = C.c_void_p()
        _check(lib().pf2_mesh_load_dat(str(path).encode(), int(fill_neighbors), C.c_double(scale), None,
                                       C.byref(h)), "pf2_mesh_load_dat")
        return cls(h)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.pf2_mesh_destroy(self.h)
            self.h = None

    def download(self, field):
        f = MESH_FIELDS[field]
        shapes = {"xy": ((self.nv, 2), np.float64), "tri": ((self.nc, 3), np.int32),
                  "area": ((self.nc,), np.float64), "inv_jacobi": ((self.nc, 4), np.float64),
                  "neighbor_offsets": ((self.nc + 1,), np.int32),
                  "neighbor_indices": ((max(self.n_neighbor_entries, 0),), np.int32),
                  "edge_ids": ((self.nc, 3), np.int32)}
        shape, dt = shapes[field]
        out = np.empty(shape, dt)
        if out.size:
            _check(lib().pf2_mesh_download(self.h, f, out.ctypes.data_as(C.c_void_p)), "pf2_mesh_download")
        return out

    def set_channel_boundary_ids(self, lx, ly, cylinder=None):
        cx, cy, r = cylinder if cylinder is not None else (0.0, 0.0, 0.0)
        _check(lib().pf2_mesh_set_channel_boundary_ids(self.h, C.c_double(lx), C.c_double(ly),
                                                       int(cylinder is not None), C.c_double(cx), C.c_double(cy),
                                                       C.c_double(r), _stream()), "pf2_mesh_set_channel_boundary_ids")


class Mesh3D:
    """Mesh3D (src/mesh_3d.cuh): vertices, tetrahedra, volumes, inverse Jacobians,
    face-sharing neighbour lists and the node graph's CSR pattern, built on the device."""

    FIELDS = {"xyz": 0, "tet": 1, "volume": 2, "inv_jacobi": 3, "neighbor_offsets": 4, "neighbor_indices": 5}

    def __init__(self, handle):
        self.h = handle
        nv, nc, nn = C.c_int(), C.c_int(), C.c_int()
        _check(lib().pf2_mesh3d_sizes(self.h, C.byref(nv), C.byref(nc), C.byref(nn)), "pf2_mesh3d_sizes")
        self.nv, self.nc, self.n_neighbor_entries = nv.value, nc.value, nn.value

    @classmethod
    def from_arrays(cls, xyz, tet, fill_neighbors=True):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        tet = np.ascontiguousarray(tet, dtype=np.int32)
        h = C.c_void_p()
        _check(lib().pf2_mesh3d_create(int(xyz.shape[0]), xyz.ctypes.data_as(C.c_void_p), int(tet.shape[0]),
                                       tet.ctypes.data_as(C.c_void_p), int(fill_neighbors), None, C.byref(h)),
               "pf2_mesh3d_create")
        return cls(h)

    @classmethod
    def load_dat(cls, path, fill_neighbors=True, scale=1.0):
        h = C.c_void_p()
        _check(lib().pf2_mesh3d_load_dat(str(path).encode(), int(fill_neighbors), C.c_double(scale), None,
                                         C.byref(h)), "pf2_mesh3d_load_dat")
        return cls(h)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.pf2_mesh3d_destroy(self.h)
            self.h = None

    def download(self, field):
        shapes = {"xyz": ((self.nv, 3), np.float64), "tet": ((self.nc, 4), np.int32),
                  "volume": ((self.nc,), np.float64), "inv_jacobi": ((self.nc, 3, 3), np.float64),
                  "neighbor_offsets": ((self.nc + 1,), np.int32),
                  "neighbor_indices": ((max(self.n_neighbor_entries, 0),), np.int32)}
        shape, dt = shapes[field]
        out = np.empty(shape, dt)
        if out.size:
            _check(lib().pf2_mesh3d_download(self.h, self.FIELDS[field], out.ctypes.data_as(C.c_void_p)),
                   "pf2_mesh3d_download")
        return out


class SparseMatrixCSR:
    """SparseMatrixCSR (src/linear_algebra/sparse_matrix.cuh) on the mesh's pattern
    (a Mesh2D or a Mesh3D)."""

    def __init__(self, mesh):
        self.mesh = mesh
        self.h = C.c_void_p()
        if isinstance(mesh, Mesh3D):
            _check(lib().pf2_csr_create_3d(mesh.h, C.byref(self.h)), "pf2_csr_create_3d")
        else:
            _check(lib().pf2_csr_create(mesh.h, C.byref(self.h)), "pf2_csr_create")
        n, nnz = C.c_int(), C.c_int()
        _check(lib().pf2_csr_sizes(self.h, C.byref(n), C.byref(nnz)), "pf2_csr_sizes")
        self.rows, self.nnz = n.value, nnz.value

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None and not getattr(self, "borrowed", False):
            _lib.pf2_csr_destroy(self.h)
            self.h = None

    def download(self):
        rp = np.empty(self.rows + 1, np.int32)
        col = np.empty(self.nnz, np.int32)
        val = np.empty(self.nnz, np.float64)
        _check(lib().pf2_csr_download(self.h, rp.ctypes.data_as(C.c_void_p), col.ctypes.data_as(C.c_void_p),
                                      val.ctypes.data_as(C.c_void_p)), "pf2_csr_download")
        return rp, col, val

    def upload_values(self, val):
        val = np.ascontiguousarray(val, dtype=np.float64)
        _check(lib().pf2_csr_upload_values(self.h, val.ctypes.data_as(C.c_void_p)), "pf2_csr_upload_values")

    def clear_values(self):
        _check(lib().pf2_csr_clear_values(self.h, _stream()), "pf2_csr_clear_values")


class DirichletBCs:
    """DirichletBCs (src/Dirichlet_bcs.cuh): setupDirichletBCs + setupNodeMap."""

    def __init__(self, n_nodes, nodes):
        arr = (DirichletNode * max(len(nodes), 1))()
        for k, (i, g) in enumerate(nodes):
            arr[k].node = int(i)
            arr[k].value = float(g)
        self.n = len(nodes)
        self.h = C.c_void_p()
        _check(lib().pf2_bc_create(int(n_nodes), len(nodes), arr, C.byref(self.h)), "pf2_bc_create")

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.pf2_bc_destroy(self.h)
            self.h = None

    def apply(self, A: SparseMatrixCSR, rhs):
        _check(lib().pf2_bc_apply(self.h, A.h, _dev(rhs), _stream()), "pf2_bc_apply")


def assemble_poisson(mesh, A, rhs, rhs_kind=RHS_SINSIN, lam=1.0, bc=None):
    """PoissonIntegrator::assembleSystem (cases/Poisson2D/main.cu:70-85), optionally
    with the Dirichlet rule fused."""
    _check(lib().pf2_assemble_poisson(mesh.h, A.h, _dev(rhs), int(rhs_kind), C.c_double(lam),
                                      bc.h if bc is not None else None, _stream()), "pf2_assemble_poisson")


def assemble_poisson_3d(mesh, A, rhs, rhs_kind=RHS3D_GAUSSIAN, lam=0.5, bc=None):
    """PoissonIntegrator::assembleSystem of cases/Poisson3D/main.cu:79-85 (lambda 0.5
    and the Gaussian rhs there), then the Dirichlet rule when bc is given."""
    _check(lib().pf2_assemble_poisson_3d(mesh.h, A.h, _dev(rhs), int(rhs_kind), C.c_double(lam),
                                         bc.h if bc is not None else None, _stream()), "pf2_assemble_poisson_3d")


def assemble_velocity_prediction(mesh, p, ux, uy, uxo, uyo, pold, Ax, Ay, rx, ry, bcx=None, bcy=None):
    _check(lib().pf2_assemble_velocity_prediction(mesh.h, C.byref(p), _dev(ux), _dev(uy), _dev(uxo), _dev(uyo),
                                                  _dev(pold), Ax.h, Ay.h, _dev(rx), _dev(ry),
                                                  bcx.h if bcx else None, bcy.h if bcy else None, _stream()),
           "pf2_assemble_velocity_prediction")


def assemble_pressure(mesh, p, px, py, pold, A, rhs, bc=None):
    _check(lib().pf2_assemble_pressure(mesh.h, C.byref(p), _dev(px), _dev(py), _dev(pold), A.h, _dev(rhs),
                                       bc.h if bc else None, _stream()), "pf2_assemble_pressure")


def assemble_velocity_correction(mesh, p, px, py, pres, pold, Ax, Ay, rx, ry, bcx=None, bcy=None):
    _check(lib().pf2_assemble_velocity_correction(mesh.h, C.byref(p), _dev(px), _dev(py), _dev(pres), _dev(pold),
                                                  Ax.h, Ay.h, _dev(rx), _dev(ry), bcx.h if bcx else None,
                                                  bcy.h if bcy else None, _stream()),
           "pf2_assemble_velocity_correction")


def prediction_bc_values(mesh, p, source: DirichletBCs, target: DirichletBCs, pres, pold, component):
    _check(lib().pf2_prediction_bc_values(mesh.h, C.byref(p), source.h, target.h, _dev(pres), _dev(pold),
                                          int(component), _stream()), "pf2_prediction_bc_values")


def bc_values(bc: DirichletBCs):
    """Current boundary values of a set, as a device tensor."""
    import torch
    out = torch.empty(max(bc.n, 1), dtype=torch.float64, device="cuda")
    _check(lib().pf2_bc_get_values(bc.h, _dev(out), _stream()), "pf2_bc_get_values")
    return out[: bc.n]


def body_loads(mesh, p, ux, uy, pres, center=(0.2, 0.2)):
    out = (C.c_double * 2)()
    _check(lib().pf2_body_loads(mesh.h, C.byref(p), C.c_double(center[0]), C.c_double(center[1]), _dev(ux),
                                _dev(uy), _dev(pres), out, _stream()), "pf2_body_loads")
    return out[0], out[1]


def export_vtu(mesh, path, fields):
    """DataExport::exportToVTK / DataExport3D::exportToVTK: the mesh and node fields
    ({name: device tensor}) as VTU."""
    names = list(fields)
    arr_n = (C.c_char_p * max(len(names), 1))(*[n.encode() for n in names])
    arr_f = (C.c_void_p * max(len(names), 1))(*[_dev(fields[n]) for n in names])
    if isinstance(mesh, Mesh3D):
        _check(lib().pf2_export_vtu_3d(mesh.h, str(path).encode(), len(names), arr_n, arr_f, _stream()),
               "pf2_export_vtu_3d")
    else:
        _check(lib().pf2_export_vtu(mesh.h, str(path).encode(), len(names), arr_n, arr_f, _stream()),
               "pf2_export_vtu")


def spmv(A, x, y):
    _check(lib().pf2_spmv(A.h, _dev(x), _dev(y), _stream()), "pf2_spmv")


class LinearSolver:
    """SolverCG / SolverGMRES (src/linear_algebra/linear_solver.cuh) with a
    preconditioner (preconditioners.cuh)."""

    def __init__(self, A: SparseMatrixCSR, kind="cg", precond="jacobi", tol=1e-8, maxit=1000,
                 criterion=CRITERION_ABS, precision=PRECISION_FP64, restart=0, ordering=0, orthogonalization=0,
                 cg_variant=0):
        o = SolverOptions()
        o.kind = {"gmres": SOLVER_GMRES, "bicgstab": SOLVER_BICGSTAB}.get(kind, SOLVER_CG)
        o.precond = PRECOND[precond] if isinstance(precond, str) else int(precond)
        o.tolerance = tol
        o.max_iterations = maxit
        o.criterion = criterion
        o.precision = precision
        o.restart = restart
        o.ordering = ordering
        o.orthogonalization = orthogonalization
        o.cg_variant = cg_variant
        self.h = C.c_void_p()
        _check(lib().pf2_solver_create(A.h, C.byref(o), C.byref(self.h)), "pf2_solver_create")

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.pf2_solver_destroy(self.h)
            self.h = None

    def solve(self, A, x, b, check=True):
        info = SolveInfo()
        st = lib().pf2_solver_solve(self.h, A.h, _dev(x), _dev(b), C.byref(info), _stream())
        if check and st not in (OK, NOT_CONVERGED):
            _check(st, "pf2_solver_solve")
        return info

    def setup(self, A):
        _check(lib().pf2_solver_setup(self.h, A.h, _stream()), "pf2_solver_setup")

    def apply_preconditioner(self, dst, src):
        _check(lib().pf2_precond_apply(self.h, _dev(dst), _dev(src), _stream()), "pf2_precond_apply")


class ParticleHandler2D:
    """ParticleHandler2D (src/particles/particle_handler_2d.cuh)."""

    FIELDS = ("x", "y", "l0", "l1", "l2", "u", "v")

    def __init__(self, mesh: Mesh2D, level, capacity_factor=2.0, handle=None):
        self.mesh = mesh
        self.owned = handle is None
        if handle is None:
            self.h = C.c_void_p()
            _check(lib().pf2_particles_create(mesh.h, int(level), C.c_double(capacity_factor), C.byref(self.h)),
                   "pf2_particles_create")
        else:
            self.h = handle

    def __del__(self):
        if getattr(self, "h", None) and self.owned and _lib is not None:
            _lib.pf2_particles_destroy(self.h)
            self.h = None

    def seed(self):
        _check(lib().pf2_particles_seed(self.h, _stream()), "pf2_particles_seed")

    def init_velocity(self, ux, uy):
        _check(lib().pf2_particles_init_velocity(self.h, _dev(ux), _dev(uy), _stream()), "init_velocity")

    def advect(self, ux, uy, dt, substeps):
        _check(lib().pf2_particles_advect(self.h, _dev(ux), _dev(uy), C.c_double(dt), int(substeps), _stream()),
               "pf2_particles_advect")

    def correct(self, ux, uy, uxo, uyo):
        _check(lib().pf2_particles_correct(self.h, _dev(ux), _dev(uy), _dev(uxo), _dev(uyo), _stream()),
               "pf2_particles_correct")

    def project(self, ux, uy):
        _check(lib().pf2_particles_project(self.h, _dev(ux), _dev(uy), _stream()), "pf2_particles_project")

    def count(self):
        n = C.c_int()
        _check(lib().pf2_particles_count(self.h, C.byref(n)), "pf2_particles_count")
        return n.value

    def export_vtu(self, path):
        """DataExport::exportParticlesToVTK: positions and velocities as VTU vertices."""
        _check(lib().pf2_export_particles_vtu(self.h, str(path).encode()), "pf2_export_particles_vtu")

    def download(self):
        n = self.count()
        arr = {k: np.empty(n, np.float64) for k in self.FIELDS}
        cell = np.empty(n, np.int32)
        _check(lib().pf2_particles_download(self.h, *[arr[k].ctypes.data_as(C.c_void_p) for k in self.FIELDS],
                                            cell.ctypes.data_as(C.c_void_p)), "pf2_particles_download")
        arr["cell"] = cell
        return arr

    def reserve(self, capacity):
        """Grows the particle buffers to `capacity` particles, keeping the particles."""
        _check(lib().pf2_particles_reserve(self.h, C.c_longlong(int(capacity))), "pf2_particles_reserve")

    def save(self, path):
        """Checkpoint of the particle state (pf2_particles_save)."""
        _check(lib().pf2_particles_save(self.h, str(path).encode()), "pf2_particles_save")

    def load(self, path):
        """Restores a checkpoint written by save() for the same mesh and level."""
        _check(lib().pf2_particles_load(self.h, str(path).encode()), "pf2_particles_load")

    def upload(self, P):
        n = int(P["cell"].size)
        a = {k: np.ascontiguousarray(P[k], dtype=np.float64) for k in self.FIELDS}
        cell = np.ascontiguousarray(P["cell"], dtype=np.int32)
        _check(lib().pf2_particles_upload(self.h, n, *[a[k].ctypes.data_as(C.c_void_p) for k in self.FIELDS],
                                          cell.ctypes.data_as(C.c_void_p)), "pf2_particles_upload")


class FlowEngine:
    """One PFEM-2 time step of the channel drivers (cases/Cylinder2D/main.cu:793-880)."""

    def __init__(self, mesh: Mesh2D, params: Params, bc_u, bc_v, bc_p, capacity_factor=2.0):
        self.mesh = mesh
        self.params = params

        def arr(b):
            a = (DirichletNode * max(len(b), 1))()
            for k, (i, g) in enumerate(b):
                a[k].node = int(i)
                a[k].value = float(g)
            return len(b), a

        nu, au = arr(bc_u)
        nv, av = arr(bc_v)
        npr, ap = arr(bc_p)
        self.h = C.c_void_p()
        _check(lib().pf2_flow_create(mesh.h, C.byref(params), nu, au, nv, av, npr, ap, C.c_double(capacity_factor),
                                     C.byref(self.h)), "pf2_flow_create")
        ph = C.c_void_p()
        _check(lib().pf2_flow_particles(self.h, C.byref(ph)), "pf2_flow_particles")
        self.particles = ParticleHandler2D(mesh, params.level, handle=ph)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.pf2_flow_destroy(self.h)
            self.h = None

    def seed(self):
        _check(lib().pf2_flow_seed(self.h, _stream()), "pf2_flow_seed")

    def step(self):
        _check(lib().pf2_flow_step(self.h, _stream()), "pf2_flow_step")

    def system(self, which):
        """(matrix, rhs device pointer) of one of the flow's systems (2 = pressure)."""
        a, r = C.c_void_p(), C.c_void_p()
        _check(lib().pf2_flow_system(self.h, int(which), C.byref(a), C.byref(r)), "pf2_flow_system")
        A = SparseMatrixCSR.__new__(SparseMatrixCSR)
        A.mesh, A.h = self.mesh, a
        n, nnz = C.c_int(), C.c_int()
        _check(lib().pf2_csr_sizes(a, C.byref(n), C.byref(nnz)), "pf2_csr_sizes")
        A.rows, A.nnz = n.value, nnz.value
        A.borrowed = True
        return A, r.value

    def set_graphs(self, enable):
        _check(lib().pf2_flow_set_graphs(self.h, int(enable)), "pf2_flow_set_graphs")

    def save(self, path):
        """Checkpoint between steps (pf2_flow_save)."""
        _check(lib().pf2_flow_save(self.h, str(path).encode(), _stream()), "pf2_flow_save")

    def load(self, path):
        """Restores a checkpoint into an engine built with the same mesh, parameters and
        Dirichlet sets; the following steps repeat the saved run's."""
        _check(lib().pf2_flow_load(self.h, str(path).encode(), _stream()), "pf2_flow_load")

    def info(self):
        info = StepInfo()
        _check(lib().pf2_flow_step_info(self.h, C.byref(info)), "pf2_flow_step_info")
        return info

    def field_ptr(self, name):
        p = C.c_void_p()
        _check(lib().pf2_flow_field(self.h, FIELDS[name], C.byref(p)), "pf2_flow_field")
        return p.value

    def field(self, name):
        """Host copy of a node field."""
        out = np.empty(self.mesh.nv, np.float64)
        _check(lib().pf2_flow_download_field(self.h, FIELDS[name], out.ctypes.data_as(C.c_void_p)),
               "pf2_flow_download_field")
        return out

    def set_field(self, name, values):
        a = np.ascontiguousarray(values, dtype=np.float64)
        _check(lib().pf2_flow_upload_field(self.h, FIELDS[name], a.ctypes.data_as(C.c_void_p)),
               "pf2_flow_upload_field")


class LearnedGuess:
    """The message-passing network of the learned initial guess (pf2_mpnn_*)."""

    IN, H, LAYERS = 5, 64, 3

    def __init__(self, mesh: Mesh2D, seed=0):
        self.mesh = mesh
        self.h = C.c_void_p()
        _check(lib().pf2_mpnn_create(mesh.h, C.c_ulonglong(seed), C.byref(self.h)), "pf2_mpnn_create")
        self.n_params = lib().pf2_mpnn_param_count()

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.pf2_mpnn_destroy(self.h)
            self.h = None

    def params(self):
        p = np.empty(self.n_params, np.float32)
        _check(lib().pf2_mpnn_get_params(self.h, p.ctypes.data_as(C.c_void_p), None), "pf2_mpnn_get_params")
        return p

    def grad(self):
        g = np.empty(self.n_params, np.float32)
        _check(lib().pf2_mpnn_get_params(self.h, None, g.ctypes.data_as(C.c_void_p)), "pf2_mpnn_get_params")
        return g

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(lib().pf2_mpnn_set_params(self.h, p.ctypes.data_as(C.c_void_p)), "pf2_mpnn_set_params")

    def save(self, path):
        _check(lib().pf2_mpnn_save(self.h, str(path).encode()), "pf2_mpnn_save")

    def load(self, path):
        _check(lib().pf2_mpnn_load(self.h, str(path).encode()), "pf2_mpnn_load")

    def forward(self, feat, y):
        _check(lib().pf2_mpnn_forward(self.h, _dev(feat), _dev(y), _stream()), "pf2_mpnn_forward")

    def train_step(self, feat, target, lr=1e-3, apply=True):
        loss = C.c_double()
        _check(lib().pf2_mpnn_train_step(self.h, _dev(feat), _dev(target), C.c_float(lr), int(apply),
                                         C.byref(loss), _stream()), "pf2_mpnn_train_step")
        return loss.value
