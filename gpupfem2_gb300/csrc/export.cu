// export.cu - VTU output of node fields (2D and 3D meshes) and particles.
//
// DataExport::exportToVTK / exportParticlesToVTK (src/data_export.cu:17-171): an ASCII
// VTK UnstructuredGrid with the mesh (points, triangles as VTK type 5) and one Float32
// point-data array per registered node field, or the particles as VTK vertices (type 1)
// with their velocity.  The element layout is the reference's, so files load in the
// same ParaView pipelines; values are written with 9 significant digits (every Float32
// value round-trips) instead of the stream default of 6.
#include <cstdio>
#include <vector>

#include "common.cuh"
#include "internal.cuh"

using namespace pf2;

namespace {

struct File {
    FILE* f = nullptr;
    explicit File(const char* path) : f(fopen(path, "w")) {}
    ~File() {
        if (f) fclose(f);
    }
};

void header(FILE* f, long long points, long long cells) {
    fprintf(f, "<?xml version=\"1.0\" ?> \n");
    fprintf(f, "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n");
    fprintf(f, "  <UnstructuredGrid>\n");
    fprintf(f, "    <Piece NumberOfPoints=\"%lld\" NumberOfCells=\"%lld\">\n", points, cells);
}

void footer(FILE* f) {
    fprintf(f, "    </Piece>\n");
    fprintf(f, "  </UnstructuredGrid>\n");
    fprintf(f, "</VTKFile>\n");
}

}  // namespace

extern "C" {

pf2_status pf2_export_vtu(const pf2_mesh* m, const char* path, int nfields, const char* const* names,
                          const double* const* fields, void* stream) {
    PF2_REQUIRE(m && path && nfields >= 0 && (nfields == 0 || (names && fields)), PF2_BAD_INPUT, "null argument");
    cudaStream_t st = as_stream(stream);
    const int nv = m->nv, nc = m->nc;
    std::vector<std::vector<double>> host(nfields, std::vector<double>(nv));
    for (int k = 0; k < nfields; ++k) {
        PF2_REQUIRE(names[k] && fields[k], PF2_BAD_INPUT, "field %d: null name or data", k);
        PF2_CUDA(cudaMemcpyAsync(host[k].data(), fields[k], sizeof(double) * nv, cudaMemcpyDeviceToHost, st));
    }
    PF2_CUDA(cudaStreamSynchronize(st));
    File out(path);
    PF2_REQUIRE(out.f, PF2_IO_ERROR, "cannot open %s for writing", path);
    FILE* f = out.f;
    header(f, nv, nc);
    fprintf(f, "      <Points>\n");
    fprintf(f, "        <DataArray type=\"Float32\" NumberOfComponents=\"3\" Format=\"ascii\">\n");
    for (int i = 0; i < nv; ++i) fprintf(f, "        %.9g %.9g 0.0\n", m->h_xy[2 * i], m->h_xy[2 * i + 1]);
    fprintf(f, "        </DataArray>\n");
    fprintf(f, "      </Points>\n");
    fprintf(f, "      <Cells>\n");
    fprintf(f, "        <DataArray type=\"Int32\" Name=\"connectivity\" Format=\"ascii\">\n          ");
    for (int c = 0; c < nc; ++c) fprintf(f, "%d %d %d ", m->h_tri[3 * c], m->h_tri[3 * c + 1], m->h_tri[3 * c + 2]);
    fprintf(f, "\n        </DataArray>\n");
    fprintf(f, "        <DataArray type=\"Int32\" Name=\"offsets\" Format=\"ascii\">\n          ");
    for (int c = 0; c < nc; ++c) fprintf(f, "%lld ", 3ll * (c + 1));
    fprintf(f, "\n        </DataArray>\n");
    fprintf(f, "        <DataArray type=\"UInt8\" Name=\"types\" Format=\"ascii\">\n          ");
    for (int c = 0; c < nc; ++c) fprintf(f, "5 ");
    fprintf(f, "\n        </DataArray>\n");
    fprintf(f, "      </Cells>\n");
    if (nfields > 0) {
        fprintf(f, "      <PointData Scalars=\"scalars\">\n");
        for (int k = 0; k < nfields; ++k) {
            fprintf(f, "        <DataArray type=\"Float32\" Name=\"%s\" Format=\"ascii\">\n        ", names[k]);
            for (int i = 0; i < nv; ++i) fprintf(f, "%.9g  ", host[k][i]);
            fprintf(f, "\n        </DataArray>\n");
        }
        fprintf(f, "      </PointData>\n");
    }
    footer(f);
    PF2_REQUIRE(!ferror(f), PF2_IO_ERROR, "write error on %s", path);
    return PF2_OK;
}

// DataExport3D::exportToVTK (src/data_export_3d.cu:15-93): the same document with
// three coordinates per point and tetrahedra (VTK type 10).
pf2_status pf2_export_vtu_3d(const pf2_mesh3d* m, const char* path, int nfields, const char* const* names,
                             const double* const* fields, void* stream) {
    PF2_REQUIRE(m && path && nfields >= 0 && (nfields == 0 || (names && fields)), PF2_BAD_INPUT, "null argument");
    cudaStream_t st = as_stream(stream);
    const int nv = m->nv, nc = m->nc;
    std::vector<std::vector<double>> host(nfields, std::vector<double>(nv));
    for (int k = 0; k < nfields; ++k) {
        PF2_REQUIRE(names[k] && fields[k], PF2_BAD_INPUT, "field %d: null name or data", k);
        PF2_CUDA(cudaMemcpyAsync(host[k].data(), fields[k], sizeof(double) * nv, cudaMemcpyDeviceToHost, st));
    }
    PF2_CUDA(cudaStreamSynchronize(st));
    File out(path);
    PF2_REQUIRE(out.f, PF2_IO_ERROR, "cannot open %s for writing", path);
    FILE* f = out.f;
    header(f, nv, nc);
    fprintf(f, "      <Points>\n");
    fprintf(f, "        <DataArray type=\"Float32\" NumberOfComponents=\"3\" Format=\"ascii\">\n");
    for (int i = 0; i < nv; ++i)
        fprintf(f, "        %.9g %.9g %.9g\n", m->h_xyz[3 * i], m->h_xyz[3 * i + 1], m->h_xyz[3 * i + 2]);
    fprintf(f, "        </DataArray>\n");
    fprintf(f, "      </Points>\n");
    fprintf(f, "      <Cells>\n");
    fprintf(f, "        <DataArray type=\"Int32\" Name=\"connectivity\" Format=\"ascii\">\n          ");
    for (int c = 0; c < nc; ++c)
        fprintf(f, "%d %d %d %d ", m->h_tet[4 * c], m->h_tet[4 * c + 1], m->h_tet[4 * c + 2], m->h_tet[4 * c + 3]);
    fprintf(f, "\n        </DataArray>\n");
    fprintf(f, "        <DataArray type=\"Int32\" Name=\"offsets\" Format=\"ascii\">\n          ");
    for (int c = 0; c < nc; ++c) fprintf(f, "%lld ", 4ll * (c + 1));
    fprintf(f, "\n        </DataArray>\n");
    fprintf(f, "        <DataArray type=\"UInt8\" Name=\"types\" Format=\"ascii\">\n          ");
    for (int c = 0; c < nc; ++c) fprintf(f, "10 ");
    fprintf(f, "\n        </DataArray>\n");
    fprintf(f, "      </Cells>\n");
    if (nfields > 0) {
        fprintf(f, "      <PointData Scalars=\"scalars\">\n");
        for (int k = 0; k < nfields; ++k) {
            fprintf(f, "        <DataArray type=\"Float32\" Name=\"%s\" Format=\"ascii\">\n        ", names[k]);
            for (int i = 0; i < nv; ++i) fprintf(f, "%.9g  ", host[k][i]);
            fprintf(f, "\n        </DataArray>\n");
        }
        fprintf(f, "      </PointData>\n");
    }
    footer(f);
    PF2_REQUIRE(!ferror(f), PF2_IO_ERROR, "write error on %s", path);
    return PF2_OK;
}

pf2_status pf2_export_particles_vtu(const pf2_particles* ph, const char* path) {
    PF2_REQUIRE(ph && path, PF2_BAD_INPUT, "null argument");
    int n = 0;
    PF2_TRY(pf2_particles_count(const_cast<pf2_particles*>(ph), &n));
    std::vector<double> x(n), y(n), u(n), v(n);
    PF2_TRY(pf2_particles_download(ph, x.data(), y.data(), nullptr, nullptr, nullptr, u.data(), v.data(), nullptr));
    File out(path);
    PF2_REQUIRE(out.f, PF2_IO_ERROR, "cannot open %s for writing", path);
    FILE* f = out.f;
    header(f, n, n);
    fprintf(f, "      <Points>\n");
    fprintf(f, "        <DataArray type=\"Float32\" NumberOfComponents=\"3\" Format=\"ascii\">\n");
    for (int p = 0; p < n; ++p) fprintf(f, "          %.9g %.9g 0.0\n", x[p], y[p]);
    fprintf(f, "        </DataArray>\n");
    fprintf(f, "      </Points>\n");
    fprintf(f, "      <Cells>\n");
    fprintf(f, "        <DataArray type=\"Int32\" Name=\"connectivity\" Format=\"ascii\">\n        ");
    for (int p = 0; p < n; ++p) fprintf(f, "  %d", p);
    fprintf(f, "\n        </DataArray>\n");
    fprintf(f, "        <DataArray type=\"Int32\" Name=\"offsets\" Format=\"ascii\">\n        ");
    for (int p = 0; p < n; ++p) fprintf(f, "  %d", p + 1);
    fprintf(f, "\n        </DataArray>\n");
    fprintf(f, "        <DataArray type=\"Int32\" Name=\"types\" Format=\"ascii\">\n        ");
    for (int p = 0; p < n; ++p) fprintf(f, "  1");
    fprintf(f, "\n        </DataArray>\n");
    fprintf(f, "      </Cells>\n");
    fprintf(f, "      <PointData Scalars=\"scalars\">\n");
    fprintf(f, "        <DataArray type=\"Float32\" Name=\"velocity\" NumberOfComponents=\"3\" Format=\"ascii\">\n");
    for (int p = 0; p < n; ++p) fprintf(f, "          %.9g %.9g 0.0\n", u[p], v[p]);
    fprintf(f, "        </DataArray>\n");
    fprintf(f, "      </PointData>\n");
    footer(f);
    PF2_REQUIRE(!ferror(f), PF2_IO_ERROR, "write error on %s", path);
    return PF2_OK;
}

}  // extern "C"
