"""The 3D path against the reference's own GPU kernels (mesh_3d.cu and
cases/Poisson3D/main.cu, compiled from the reference sources by oracle/build_ref.sh and
launched through tests/refgpu.py) on the same inputs: cell volumes and inverse
Jacobians, the face-neighbour kernel and the Poisson3D assembly kernel.

The reference computes the geometry with its own grouping of the products and sums the
assembly with atomics, so both agree to rounding, not bit for bit.  Its neighbour kernel
(kFindNeighbors, mesh_3d.cu:37-82) compares the batch-local index of a candidate with
the global index of the cell, so for a cell c < 1024 it skips the candidates
c + 1024 m (m >= 1) of later batches: its lists are the face-sharing lists (which the
engine builds) minus exactly those pairs."""
import ctypes as C

import numpy as np
import pytest
import torch

import gpupfem2_gb300 as g
from gpupfem2_gb300 import meshgen as mg
from oracle import oracle as O
from tests import refgpu as R
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

if not R.available_3d():
    pytest.skip("reference 3D kernels not built (oracle/build_ref.sh needs the reference tree)",
                allow_module_level=True)

BATCH = 1024  # gpuThreadsMax, src/common/cuda_helper.cuh:18


@pytest.fixture(scope="module")
def mod(cuda):
    return R.RefModule("ref_poisson3d.cubin", names="ref_kernels3d.names")


def ref_geometry(mod, xyz, tet):
    nc = tet.shape[0]
    v = R.dev(np.ascontiguousarray(xyz, np.float64))  # Point3 = double3, 24-byte stride
    c = R.dev(np.ascontiguousarray(tet, np.uint32))   # uint4
    vol = torch.zeros(nc, dtype=torch.float64, device="cuda")
    inv = torch.zeros(nc * R.MAT3.itemsize, dtype=torch.uint8, device="cuda")
    mod.launch("kCalculateCellVolume", nc, C.c_int(nc), v, c, vol)
    mod.launch("kCalculateInvJacobi", nc, C.c_int(nc), v, c, inv)
    torch.cuda.synchronize()
    return vol.cpu().numpy(), R.host(inv, R.MAT3)["m"].reshape(nc, 3, 3), v, c, inv


def test_geometry_matches_reference_kernels(mod):
    xyz, tet = mg.box_tets(12, 6, 4)
    vol, inv, *_ = ref_geometry(mod, xyz, tet)
    m = g.Mesh3D.from_arrays(xyz, tet)
    assert rel_err(m.download("volume"), vol) < 1e-14
    assert rel_err(m.download("inv_jacobi"), inv) < 1e-13


def ref_neighbours(mod, tet):
    nc = tet.shape[0]
    c = R.dev(np.ascontiguousarray(tet, np.uint32))
    grid = (nc + BATCH - 1) // BATCH
    # the kernel reads offsets[idx] for every thread of the last block: pad to the grid
    off = torch.zeros(grid * BATCH + 1, dtype=torch.int32, device="cuda")
    mod.launch("kFindNeighbors", nc, C.c_int(nc), c, off, None, block=BATCH)
    torch.cuda.synchronize()
    counts = off[1:nc + 1].cpu().numpy()
    offsets = np.zeros(grid * BATCH + 1, np.int32)
    offsets[1:nc + 1] = np.cumsum(counts)
    total = int(offsets[nc])
    offsets[nc + 1:] = total
    off_d = torch.tensor(offsets, device="cuda")
    idx = torch.full((max(total, 1),), -1, dtype=torch.int32, device="cuda")
    mod.launch("kFindNeighbors", nc, C.c_int(nc), c, off_d, idx, block=BATCH)
    torch.cuda.synchronize()
    return offsets[:nc + 1], idx.cpu().numpy()[:total]


def test_neighbours_against_reference_kernel(mod):
    xyz, tet = mg.box_tets(16, 8, 6)  # 4,608 cells: five batches of the reference kernel
    nc = tet.shape[0]
    # cells in a shuffled order, so that some face neighbours sit 1024 m apart (4 pairs)
    tet = tet[np.random.default_rng(4).permutation(nc)]
    roff, ridx = ref_neighbours(mod, tet)
    m = g.Mesh3D.from_arrays(xyz, tet)
    off, idx = m.download("neighbor_offsets"), m.download("neighbor_indices")
    oo, oi = O.mesh3d_neighbors(tet)
    assert np.array_equal(off, oo) and np.array_equal(idx, oi)
    dropped = 0
    for c in range(nc):
        ours = idx[off[c]:off[c + 1]].tolist()
        ref = ridx[roff[c]:roff[c + 1]].tolist()
        want = [d for d in ours if not (c < BATCH and d >= BATCH and d % BATCH == c)]
        assert ref == want, c
        dropped += len(ours) - len(want)
    assert dropped > 0  # the mesh does exercise the skipped pairs


def test_poisson3d_assembly_matches_reference_kernel(mod):
    xyz, tet = mg.box_tets(12, 6, 4)
    nc = tet.shape[0]
    vol, inv, v, c, inv_d = ref_geometry(mod, xyz, tet)
    m = g.Mesh3D.from_arrays(xyz, tet)
    A = g.SparseMatrixCSR(m)
    rp, col, _ = A.download()
    q, w = O.cell_quadrature_3d()
    table = np.zeros(31, R.GAUSS3D)
    for k in range(q.shape[0]):
        table[k] = (q[k, 0], q[k, 1], q[k, 2], q[k, 3], w[k])
    mod.set_global("cellQuadratureFormula", table.tobytes())
    mod.set_global("cellQuadraturePointsNum", np.int32(q.shape[0]).tobytes())
    vol_d = torch.tensor(vol, device="cuda")
    rp_d, col_d = torch.tensor(rp, device="cuda"), torch.tensor(col, device="cuda")
    val = torch.zeros(col.size, dtype=torch.float64, device="cuda")
    rhs = torch.zeros(m.nv, dtype=torch.float64, device="cuda")
    mod.launch("kIntegrateOverCell", nc, C.c_int(nc), v, c, vol_d, inv_d, rp_d, col_d, val, rhs)
    torch.cuda.synchronize()
    grhs = torch.zeros(m.nv, dtype=torch.float64, device="cuda")
    g.assemble_poisson_3d(m, A, grhs, g.RHS3D_GAUSSIAN, 0.5)
    assert rel_err(A.download()[2], val.cpu().numpy()) < 1e-12
    assert rel_err(grhs.cpu().numpy(), rhs.cpu().numpy()) < 1e-12
