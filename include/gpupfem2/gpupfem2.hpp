// gpupfem2.hpp - C++ classes with the reference's names and signatures
// (andreyypopov/gpuPfem2, src/), implemented over the C ABI of pf2.h.
//
// A case driver written against the reference (cases/*/main.cu) compiles against these
// classes with two changes: velocity fields are passed as two device pointers instead of
// a device array of pointers, and assembly goes through the pf2_assemble_* entry points
// instead of the driver's own kernels.  Failures throw
// gpupfem2::Error (the reference calls exit()); solver non-convergence returns false as
// in the reference.
#pragma once

#include <cuda_runtime.h>

#include <stdexcept>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../pf2.h"

namespace gpupfem2 {

struct Error : std::runtime_error {
    pf2_status status;
    Error(pf2_status s, const std::string& what)
        : std::runtime_error(what + ": " + pf2_last_error()), status(s) {}
};

inline void check(pf2_status s, const char* what) {
    if (s != PF2_OK) throw Error(s, what);
}

// deviceVector<T> (src/common/device_vector.cuh:19-146): owning device array; move-only
// (the reference's has no copy control and double-frees on copies).
template <class T>
struct deviceVector {
    T* data = nullptr;
    int size = 0;
    deviceVector() = default;
    deviceVector(const deviceVector&) = delete;
    deviceVector& operator=(const deviceVector&) = delete;
    deviceVector(deviceVector&& o) noexcept : data(o.data), size(o.size) { o.data = nullptr; o.size = 0; }
    ~deviceVector() { if (data) cudaFree(data); }
    void allocate(int n) {
        if (data) cudaFree(data);
        data = nullptr;
        if (cudaMalloc(&data, sizeof(T) * (n > 0 ? n : 1)) != cudaSuccess) throw Error(PF2_CUDA_ERROR, "cudaMalloc");
        size = n;
    }
    void clearValues() { cudaMemset(data, 0, sizeof(T) * size); }
    std::vector<T> toHost() const {
        std::vector<T> h(size);
        cudaMemcpy(h.data(), data, sizeof(T) * size, cudaMemcpyDeviceToHost);
        return h;
    }
};

// SimulationParameters (src/parameters.cuh:6-51)
struct SimulationParameters : pf2_params {
    void setDefaultParameters() { pf2_params_default(this); }
};

// DirichletNode (src/Dirichlet_bcs.cuh:8-12)
using DirichletNode = pf2_dirichlet_node;

// Mesh2D (src/mesh_2d.cuh:11-69)
class Mesh2D {
public:
    Mesh2D() = default;
    Mesh2D(const Mesh2D&) = delete;
    Mesh2D& operator=(const Mesh2D&) = delete;
    ~Mesh2D() { pf2_mesh_destroy(m_); }

    bool loadMeshFromFile(const std::string& filename, bool fillNeighborLists = true, double scale = 1.0) {
        pf2_mesh* m = nullptr;
        if (pf2_mesh_load_dat(filename.c_str(), fillNeighborLists ? 1 : 0, scale, nullptr, &m) != PF2_OK)
            return false;
        pf2_mesh_destroy(m_);
        m_ = m;
        check(pf2_mesh_view_get(m_, &v_), "pf2_mesh_view_get");
        hostVertices_.resize(v_.nv);
        hostCells_.resize(v_.nc);
        check(pf2_mesh_download(m_, PF2_MESH_XY, hostVertices_.data()), "pf2_mesh_download");
        check(pf2_mesh_download(m_, PF2_MESH_TRI, hostCells_.data()), "pf2_mesh_download");
        return true;
    }
    int numVertices() const { return v_.nv; }
    int numCells() const { return v_.nc; }
    const double2* getVertices() const { return reinterpret_cast<const double2*>(v_.xy); }
    const int* getCells() const { return v_.tri; }
    const double* getCellArea() const { return v_.area; }
    const double* getInvJacobi() const { return v_.inv_jacobi; }
    const int* getCellNeighborsOffsets() const { return v_.neighbor_offsets; }
    const int* getCellNeighborIndices() const { return v_.neighbor_indices; }
    const int* getEdgeBoundaryIDs() const { return v_.edge_boundary_ids; }
    const std::vector<double2>& getHostVertices() const { return hostVertices_; }
    const std::vector<int3>& getHostCells() const { return hostCells_; }
    pf2_mesh* handle() const { return m_; }

private:
    pf2_mesh* m_ = nullptr;
    pf2_mesh_view v_{};
    std::vector<double2> hostVertices_;
    std::vector<int3> hostCells_;
};

// Mesh3D (src/mesh_3d.cuh:11-70): linear tetrahedra.  Vertices on the device are
// (x, y, z, 0) per vertex; the host copies keep the reference's element types.
class Mesh3D {
public:
    Mesh3D() = default;
    Mesh3D(const Mesh3D&) = delete;
    Mesh3D& operator=(const Mesh3D&) = delete;
    ~Mesh3D() { pf2_mesh3d_destroy(m_); }

    bool loadMeshFromFile(const std::string& filename, bool fillNeighborLists = true, double scale = 1.0) {
        pf2_mesh3d* m = nullptr;
        if (pf2_mesh3d_load_dat(filename.c_str(), fillNeighborLists ? 1 : 0, scale, nullptr, &m) != PF2_OK)
            return false;
        pf2_mesh3d_destroy(m_);
        m_ = m;
        check(pf2_mesh3d_view_get(m_, &v_), "pf2_mesh3d_view_get");
        hostVertices_.resize(v_.nv);
        hostCells_.resize(v_.nc);
        check(pf2_mesh3d_download(m_, PF2_MESH3D_XYZ, hostVertices_.data()), "pf2_mesh3d_download");
        check(pf2_mesh3d_download(m_, PF2_MESH3D_TET, hostCells_.data()), "pf2_mesh3d_download");
        return true;
    }
    int numVertices() const { return v_.nv; }
    int numCells() const { return v_.nc; }
    const double* getVertices() const { return v_.xyz4; }  // 4 doubles per vertex
    const int4* getCells() const { return reinterpret_cast<const int4*>(v_.tet); }
    const double* getCellVolume() const { return v_.volume; }
    const double* getInvJacobi() const { return v_.inv_jacobi; }
    const int* getCellNeighborsOffsets() const { return v_.neighbor_offsets; }
    const int* getCellNeighborIndices() const { return v_.neighbor_indices; }
    const std::vector<double3>& getHostVertices() const { return hostVertices_; }
    const std::vector<int4>& getHostCells() const { return hostCells_; }
    pf2_mesh3d* handle() const { return m_; }

private:
    pf2_mesh3d* m_ = nullptr;
    pf2_mesh3d_view v_{};
    std::vector<double3> hostVertices_;
    std::vector<int4> hostCells_;
};

// SparseMatrixCSR (src/linear_algebra/sparse_matrix.cuh:9-58)
class SparseMatrixCSR {
public:
    explicit SparseMatrixCSR(const Mesh2D& mesh) { initialize(mesh); }
    explicit SparseMatrixCSR(const Mesh3D& mesh) { initialize(mesh); }
    void initialize(const Mesh3D& mesh) {
        pf2_csr_destroy(a_);
        check(pf2_csr_create_3d(mesh.handle(), &a_), "pf2_csr_create_3d");
        check(pf2_csr_view(a_, &rp_, &col_, &val_), "pf2_csr_view");
        check(pf2_csr_sizes(a_, &rows_, &nnz_), "pf2_csr_sizes");
    }
    SparseMatrixCSR(const SparseMatrixCSR&) = delete;
    SparseMatrixCSR& operator=(const SparseMatrixCSR&) = delete;
    ~SparseMatrixCSR() { pf2_csr_destroy(a_); }
    void initialize(const Mesh2D& mesh) {
        pf2_csr_destroy(a_);
        check(pf2_csr_create(mesh.handle(), &a_), "pf2_csr_create");
        check(pf2_csr_view(a_, &rp_, &col_, &val_), "pf2_csr_view");
        check(pf2_csr_sizes(a_, &rows_, &nnz_), "pf2_csr_sizes");
    }
    int* getRowOffset() const { return const_cast<int*>(rp_); }
    int* getColIndices() const { return const_cast<int*>(col_); }
    double* getMatrixValues() const { return val_; }
    int getRows() const { return rows_; }
    int getTotalElements() const { return nnz_; }
    void clearValues() { check(pf2_csr_clear_values(a_, nullptr), "pf2_csr_clear_values"); }
    pf2_csr* handle() const { return a_; }

private:
    pf2_csr* a_ = nullptr;
    const int* rp_ = nullptr;
    const int* col_ = nullptr;
    double* val_ = nullptr;
    int rows_ = 0, nnz_ = 0;
};

// DirichletBCs (src/Dirichlet_bcs.cuh:14-29)
class DirichletBCs {
public:
    ~DirichletBCs() { pf2_bc_destroy(b_); }
    void setupDirichletBCs(const std::vector<DirichletNode>& hostBcs) { nodes_ = hostBcs; rebuild(); }
    void setupNodeMap(int n, const std::vector<DirichletNode>& hostBcs) { n_ = n; nodes_ = hostBcs; rebuild(); }
    void applyBCs(SparseMatrixCSR& matrix, deviceVector<double>& rhs) {
        ensure(matrix.getRows());
        check(pf2_bc_apply(b_, matrix.handle(), rhs.data, nullptr), "pf2_bc_apply");
    }
    pf2_bc* handle(int n) { ensure(n); return b_; }

private:
    void ensure(int n) {
        if (n_ != n) { n_ = n; rebuild(); }
    }
    void rebuild() {
        if (n_ <= 0) return;
        pf2_bc_destroy(b_);
        b_ = nullptr;
        check(pf2_bc_create(n_, (int)nodes_.size(), nodes_.data(), &b_), "pf2_bc_create");
    }
    pf2_bc* b_ = nullptr;
    int n_ = 0;
    std::vector<DirichletNode> nodes_;
};

// LinearAlgebra (src/linear_algebra/linear_algebra.h): no handles are needed.
class LinearAlgebra {};

// Preconditioner{Jacobi,ILU,IC} (src/linear_algebra/preconditioners.cuh:9-106)
class Preconditioner {
public:
    explicit Preconditioner(int kind) : kind_(kind) {}
    virtual ~Preconditioner() = default;
    int kind() const { return kind_; }

private:
    int kind_;
};
class PreconditionerJacobi : public Preconditioner {
public:
    PreconditionerJacobi(int, const LinearAlgebra*) : Preconditioner(PF2_PRECOND_JACOBI) {}
};
class PreconditionerILU : public Preconditioner {
public:
    PreconditionerILU(const SparseMatrixCSR&, const LinearAlgebra*) : Preconditioner(PF2_PRECOND_ILU) {}
};
class PreconditionerIC : public Preconditioner {
public:
    PreconditionerIC(const SparseMatrixCSR&, const LinearAlgebra*) : Preconditioner(PF2_PRECOND_IC) {}
};

// LinearSolver / SolverCG / SolverGMRES (src/linear_algebra/linear_solver.cuh:15-137)
class LinearSolver {
public:
    LinearSolver(int kind, double tolerance, int maxIterations, const LinearAlgebra*, Preconditioner* precond)
        : kind_(kind), tol_(tolerance), maxit_(maxIterations),
          precond_(precond ? precond->kind() : PF2_PRECOND_NONE) {}
    virtual ~LinearSolver() { pf2_solver_destroy(s_); }
    void init(const SparseMatrixCSR& matrix) {
        pf2_solver_options o{};
        o.kind = kind_;
        o.precond = precond_;
        o.tolerance = tol_;
        o.max_iterations = maxit_;
        o.criterion = PF2_CRITERION_ABS;
        o.precision = PF2_PRECISION_FP64;
        o.restart = 0;
        pf2_solver_destroy(s_);
        check(pf2_solver_create(matrix.handle(), &o, &s_), "pf2_solver_create");
    }
    bool solve(const SparseMatrixCSR& A, deviceVector<double>& x, const deviceVector<double>& b) {
        pf2_solve_info info{};
        const pf2_status s = pf2_solver_solve(s_, A.handle(), x.data, b.data, &info, nullptr);
        if (s != PF2_OK && s != PF2_NOT_CONVERGED) throw Error(s, "pf2_solver_solve");
        last_ = info;
        return s == PF2_OK;
    }
    const pf2_solve_info& lastInfo() const { return last_; }

private:
    int kind_;
    double tol_;
    int maxit_;
    int precond_;
    pf2_solver* s_ = nullptr;
    pf2_solve_info last_{};
};
class SolverCG : public LinearSolver {
public:
    SolverCG(double tolerance, int maxIterations, const LinearAlgebra* LA, Preconditioner* precond = nullptr)
        : LinearSolver(PF2_SOLVER_CG, tolerance, maxIterations, LA, precond) {}
};
class SolverGMRES : public LinearSolver {
public:
    SolverGMRES(double tolerance, int maxIterations, const LinearAlgebra* LA, Preconditioner* precond = nullptr)
        : LinearSolver(PF2_SOLVER_GMRES, tolerance, maxIterations, LA, precond) {}
};

// ParticleHandler2D (src/particles/particle_handler_2d.cuh:9-54); velocity fields are two
// device arrays.
class ParticleHandler2D {
public:
    ParticleHandler2D(const Mesh2D* mesh, int cellDivisionLevel, double capacityFactor = 2.0) {
        check(pf2_particles_create(mesh->handle(), cellDivisionLevel, capacityFactor, &h_), "pf2_particles_create");
    }
    ParticleHandler2D(const ParticleHandler2D&) = delete;
    ParticleHandler2D& operator=(const ParticleHandler2D&) = delete;
    ~ParticleHandler2D() { pf2_particles_destroy(h_); }
    void seedParticles() { check(pf2_particles_seed(h_, nullptr), "pf2_particles_seed"); }
    void initParticleVelocity(const double* ux, const double* uy) {
        check(pf2_particles_init_velocity(h_, ux, uy, nullptr), "pf2_particles_init_velocity");
    }
    void advectParticles(const double* ux, const double* uy, double timeStep, int particleSubsteps) {
        check(pf2_particles_advect(h_, ux, uy, timeStep, particleSubsteps, nullptr), "pf2_particles_advect");
    }
    void correctParticleVelocity(const double* ux, const double* uy, const double* uxOld, const double* uyOld) {
        check(pf2_particles_correct(h_, ux, uy, uxOld, uyOld, nullptr), "pf2_particles_correct");
    }
    void projectVelocityOntoGrid(double* ux, double* uy) {
        check(pf2_particles_project(h_, ux, uy, nullptr), "pf2_particles_project");
    }
    int getParticleCount() const {
        int n = 0;
        check(pf2_particles_count(h_, &n), "pf2_particles_count");
        return n;
    }
    // checkpoint / restart (no reference counterpart): false if the file cannot be
    // written or does not fit this handler (mesh, level, capacity)
    bool saveCheckpoint(const std::string& filename) const {
        return pf2_particles_save(h_, filename.c_str()) == PF2_OK;
    }
    bool loadCheckpoint(const std::string& filename) { return pf2_particles_load(h_, filename.c_str()) == PF2_OK; }

    pf2_particles* handle() const { return h_; }

private:
    pf2_particles* h_ = nullptr;
};

// DataExport (src/data_export.cuh:10-30): node fields registered by name, written with
// the mesh as VTU; particles as VTU vertices.
class DataExport {
public:
    explicit DataExport(const Mesh2D& mesh, const ParticleHandler2D* particleHandler = nullptr)
        : mesh_(mesh), ph_(particleHandler) {}
    void addScalarDataVector(const deviceVector<double>& dataVector, const std::string& fieldname) {
        for (auto& f : fields_)
            if (f.first == fieldname) { f.second = dataVector.data; return; }
        fields_.emplace_back(fieldname, dataVector.data);
    }
    void exportToVTK(const std::string& filename) const {
        std::vector<const char*> names;
        std::vector<const double*> data;
        for (const auto& f : fields_) {
            names.push_back(f.first.c_str());
            data.push_back(f.second);
        }
        check(pf2_export_vtu(mesh_.handle(), filename.c_str(), (int)names.size(), names.data(), data.data(), nullptr),
              "pf2_export_vtu");
    }
    void exportParticlesToVTK(const std::string& filename) const {
        if (!ph_) throw Error(PF2_BAD_INPUT, "DataExport has no particle handler");
        check(pf2_export_particles_vtu(ph_->handle(), filename.c_str()), "pf2_export_particles_vtu");
    }

private:
    const Mesh2D& mesh_;
    const ParticleHandler2D* ph_;
    std::vector<std::pair<std::string, const double*>> fields_;
};

// DataExport3D (src/data_export_3d.cuh:9-23): node fields by name (written in name
// order, as the reference's std::map), tetrahedra as VTK type 10.
class DataExport3D {
public:
    explicit DataExport3D(const Mesh3D& mesh) : mesh_(mesh) {}
    void addScalarDataVector(const deviceVector<double>& dataVector, const std::string& fieldname) {
        fields_[fieldname] = dataVector.data;
    }
    void exportToVTK(const std::string& filename) const {
        std::vector<const char*> names;
        std::vector<const double*> data;
        for (const auto& f : fields_) {
            names.push_back(f.first.c_str());
            data.push_back(f.second);
        }
        check(pf2_export_vtu_3d(mesh_.handle(), filename.c_str(), (int)names.size(), names.data(), data.data(),
                                nullptr),
              "pf2_export_vtu_3d");
    }

private:
    const Mesh3D& mesh_;
    std::map<std::string, const double*> fields_;
};

}  // namespace gpupfem2
