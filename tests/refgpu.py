"""Launches the reference's own GPU kernels (TEST INFRASTRUCTURE ONLY).

oracle/build_ref.sh compiles the reference kernels from their sources into linked
sm_103a cubins (oracle/_ref/ref_flow.cubin, ref_poisson.cubin) and lists their mangled
names (ref_kernels.names).  This module loads them into torch's CUDA context through
the driver API (libcuda via ctypes), fills their __constant__ symbols and launches
them with the reference's launch shape (256 threads, ceil(n/256) blocks) on buffers
laid out as the reference's structs.  It is the checker the parity tests compare the
engine against; nothing in the engine uses it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_DIR = os.path.join(ROOT, "oracle", "_ref")

# Particle2D (src/particles/particle_2d.cuh:6-58): ID u32, position double2 (16-aligned),
# localPosition double3, velocity double2 (16-aligned), cellID u32; 96 bytes.
PARTICLE = np.dtype({"names": ["id", "x", "y", "l0", "l1", "l2", "u", "v", "cell"],
                     "formats": ["<u4", "<f8", "<f8", "<f8", "<f8", "<f8", "<f8", "<f8", "<u4"],
                     "offsets": [0, 16, 24, 32, 40, 48, 64, 72, 80], "itemsize": 96})
# GaussPoint2D {Point3 coordinates; double weight}, GaussPoint1D {double, double}
GAUSS2D = np.dtype([("x", "<f8"), ("y", "<f8"), ("z", "<f8"), ("w", "<f8")])
GAUSS1D = np.dtype([("c", "<f8"), ("w", "<f8")])
# GaussPoint3D {Point4 coordinates (double4, 16-byte aligned); double weight}: 48 bytes;
# GenericMatrix3x3 has a virtual operator(): vtable pointer, then 9 doubles (80 bytes)
GAUSS3D = np.dtype({"names": ["x", "y", "z", "w", "weight"], "formats": ["<f8"] * 5,
                    "offsets": [0, 8, 16, 24, 32], "itemsize": 48})
MAT3 = np.dtype({"names": ["vptr", "m"], "formats": ["<u8", ("<f8", (9,))], "offsets": [0, 8], "itemsize": 80})
# DirichletNode {unsigned nodeIdx; double bcValue}
DNODE = np.dtype({"names": ["node", "value"], "formats": ["<u4", "<f8"], "offsets": [0, 8], "itemsize": 16})


class SimParams(C.Structure):
    """SimulationParameters (src/parameters.cuh:6-51), the layout the kernels read."""
    _fields_ = [("rho", C.c_double), ("mu", C.c_double), ("tFinal", C.c_double), ("dt", C.c_double),
                ("tolerance", C.c_double), ("maxIterations", C.c_int), ("simulationScheme", C.c_int),
                ("meshFileName", C.c_void_p), ("outputFrequency", C.c_int), ("particleAdvectionSubsteps", C.c_int),
                ("exportParticles", C.c_int), ("calculateLoads", C.c_int), ("bodyBoundaryID", C.c_int),
                ("thickness", C.c_double), ("meanVelocity", C.c_double)]


def available():
    return all(os.path.exists(os.path.join(REF_DIR, f))
               for f in ("ref_flow.cubin", "ref_poisson.cubin", "ref_kernels.names"))


def available_3d():
    return all(os.path.exists(os.path.join(REF_DIR, f)) for f in ("ref_poisson3d.cubin", "ref_kernels3d.names"))


_cuda = None


def _drv():
    global _cuda
    if _cuda is None:
        _cuda = C.CDLL("libcuda.so.1")
    return _cuda


def _ck(rc, what):
    if rc != 0:
        raise RuntimeError("%s failed with CUresult %d" % (what, rc))


class RefModule:
    def __init__(self, cubin, names="ref_kernels.names"):
        torch.zeros(1, device="cuda")  # torch's primary context is current
        d = _drv()
        self.mod = C.c_void_p()
        _ck(d.cuModuleLoad(C.byref(self.mod), os.path.join(REF_DIR, cubin).encode()), "cuModuleLoad")
        self.names = {}
        for line in open(os.path.join(REF_DIR, names)):
            _, base, mangled = line.split()
            self.names[base] = mangled
        self.fns = {}

    def fn(self, base):
        if base not in self.fns:
            f = C.c_void_p()
            _ck(_drv().cuModuleGetFunction(C.byref(f), self.mod, self.names[base].encode()), "cuModuleGetFunction")
            self.fns[base] = f
        return self.fns[base]

    def set_global(self, name, data: bytes):
        ptr, size = C.c_uint64(), C.c_size_t()
        _ck(_drv().cuModuleGetGlobal_v2(C.byref(ptr), C.byref(size), self.mod, name.encode()), "cuModuleGetGlobal")
        if len(data) > size.value:
            raise ValueError("%s holds %d bytes, %d given" % (name, size.value, len(data)))
        buf = C.create_string_buffer(data, len(data))
        _ck(_drv().cuMemcpyHtoD_v2(ptr, buf, C.c_size_t(len(data))), "cuMemcpyHtoD")

    def launch(self, base, n, *args, block=256):
        """kernel<<<ceil(n/block), block>>>(args...) on torch's current stream; each arg is a
        ctypes scalar (c_int, c_double) or a torch tensor (passed as its device pointer)."""
        vals = []
        for a in args:
            if isinstance(a, torch.Tensor):
                vals.append(C.c_void_p(a.data_ptr()))
            elif a is None:
                vals.append(C.c_void_p(0))
            else:
                vals.append(a)
        params = (C.c_void_p * len(vals))(*[C.cast(C.pointer(v), C.c_void_p) for v in vals])
        grid = max(1, (int(n) + block - 1) // block)
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        _ck(_drv().cuLaunchKernel(self.fn(base), grid, 1, 1, block, 1, 1, 0, stream, params, None),
            "cuLaunchKernel(%s)" % base)


def dev(a, dtype=None):
    """A device tensor holding the bytes of a numpy array."""
    a = np.ascontiguousarray(a)
    t = torch.from_numpy(a.view(np.uint8).reshape(-1).copy()).cuda()
    return t


def host(t, dtype, count=None):
    b = t.cpu().numpy().view(dtype)
    return b if count is None else b[:count]


def ptr_array(*tensors):
    """A device array of device pointers (the reference's double** / const int** arguments)."""
    return dev(np.array([t.data_ptr() for t in tensors], dtype=np.uint64))


def mesh_buffers(xy, tri):
    """vertices (Point2 = double2), cells (uint3, 12-byte stride)."""
    return dev(np.ascontiguousarray(xy, np.float64)), dev(np.ascontiguousarray(tri, np.uint32))
