// dump_ref_vtu.cu - runs the reference's VTU writers (DataExport::exportToVTK and
// exportParticlesToVTK, src/data_export.cu:17-171) on the CPU against the host-memory
// runtime stand-in (stub_cudart.c), to record their output as test fixtures (TEST
// INFRASTRUCTURE ONLY).
//
// usage: ref_vtu_dump <mesh.dat> <out_prefix>
// writes <out_prefix>.mesh.vtu with three node fields and <out_prefix>.particles.vtu with
// four particles per cell; the values follow from the vertex coordinates by the formulas
// below, so a test can rebuild them:
//   velX = 1.25 x, velY = x y - 0.5, pressure = 1 - 0.3 x + 0.2 y^2
//   particle 4c + k of cell c: weights w = (k + 1, 2, 3) / (k + 6) on the vertices
//   (position = sum w_i v_i, local position w), velocity (0.5 x, 0.25 y - 1)
#include <cstdio>
#include <string>
#include <vector>

#include "common/cuda_math.cuh"
#include "common/device_vector.cuh"
#include "mesh_2d.cuh"
#include "particles/particle_2d.cuh"
// the harness fills the particle handler's (private) particle array itself
#define private public
#include "particles/particle_handler_2d.cuh"
#undef private
#include "data_export.cuh"

int main(int argc, char** argv) {
    if (argc < 3) { fprintf(stderr, "usage: %s mesh.dat out_prefix\n", argv[0]); return 1; }
    const std::string out = argv[2];
    Mesh2D mesh;
    if (!mesh.loadMeshFromFile(argv[1])) return 1;
    const auto& hv = mesh.getHostVertices();
    const int nv = hv.size();
    const int nc = mesh.getCells().size;
    const auto& hc = mesh.getHostCells();
    deviceVector<double> vx, vy, pr;
    vx.allocate(nv);
    vy.allocate(nv);
    pr.allocate(nv);
    for (int i = 0; i < nv; ++i) {  // "device" memory is host memory under the stand-in
        vx.data[i] = 1.25 * hv[i].x;
        vy.data[i] = hv[i].x * hv[i].y - 0.5;
        pr.data[i] = 1.0 - 0.3 * hv[i].x + 0.2 * hv[i].y * hv[i].y;
    }
    ParticleHandler2D ph(&mesh, 2);
    ph.particleCount = 4 * nc;
    ph.particles.allocate(ph.particleCount);
    for (int c = 0; c < nc; ++c)
        for (int k = 0; k < 4; ++k) {
            const double w0 = (k + 1.0) / (k + 6.0), w1 = 2.0 / (k + 6.0), w2 = 3.0 / (k + 6.0);
            const Point2 a = hv[hc[c].x], b = hv[hc[c].y], d = hv[hc[c].z];
            const Point2 pos = { w0 * a.x + w1 * b.x + w2 * d.x, w0 * a.y + w1 * b.y + w2 * d.y };
            Particle2D p(pos, { w0, w1, w2 }, 4 * c + k);
            p.setCellID(c);
            p.setVelocity({ 0.5 * pos.x, 0.25 * pos.y - 1.0 });
            ph.particles.data[4 * c + k] = p;
        }
    DataExport ex(mesh, &ph);
    ex.addScalarDataVector(vx, "velX");
    ex.addScalarDataVector(vy, "velY");
    ex.addScalarDataVector(pr, "pressure");
    ex.exportToVTK(out + ".mesh.vtu");
    ex.exportParticlesToVTK(out + ".particles.vtu");
    return 0;
}
