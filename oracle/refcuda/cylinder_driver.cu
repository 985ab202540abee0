// Reference-CUDA timing driver (MEASUREMENT INFRASTRUCTURE ONLY: it runs the reference
// gpuPfem2 code, compiled from its own sources by oracle/build_ref_cuda.sh, to time the
// reference's step on this GPU; the engine never links it).
//
// The reference's Cylinder2D case (cases/Cylinder2D/main.cu) hard-codes its mesh file,
// particle level, time step and scheme inside main().  This driver compiles that file as
// it is (its main() renamed, so the case's kernels and classes -- CylinderIntegrator,
// VelocityDirichletBCs, boundaryLoadsCalculator, the __constant__ quadrature and
// parameters -- come from the reference itself) and runs the same step loop
// (main.cu:793-880) on a mesh, level, dt and scheme given on the command line:
//
//   ref_cylinder MESH.dat LEVEL DT SCHEME PRESSURE_PRECOND(jacobi|ic) WARMUP STEPS OUT.json
//
// Two departures, both outside the timed steps:
//  * Mesh2D::loadMeshFromFile is called with fillNeighborLists = false and the neighbour
//    lists are filled here from the node incidence in O(N): for each cell, every other
//    cell sharing at least one vertex, ascending.  That is the content of the reference's
//    all-pairs builder (mesh_2d.cu:107-139), which at a million cells compares ~5e11 cell
//    pairs on one host thread.
//  * The pressure solver is the case's Jacobi-CG (main.cu:769-771) or, with "ic", CG with
//    the reference's PreconditionerIC (preconditioners.cu:136-213) for the pressure alone;
//    the velocity solves keep the case's Jacobi-CG and Jacobi-GMRES.
//
// Each step is timed with the reference's own GpuTimer (common/gpu_timer.cuh), its phases
// with CUDA events on the default stream (the spans of the case's ProfilingScope calls).
// OUT.json receives the per-step times of the timed steps, the mean phase times and the
// particle count; the case's boundaryLoadsCalculator writes Forces.csv in the working
// directory as in the reference.
#include <algorithm>
#include <array>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <set>
#include <string>
#include <vector>

#include "common/cuda_math.cuh"
#include "common/device_vector.cuh"
// the driver fills Mesh2D's (private) neighbour arrays itself
#define private public
#include "mesh_2d.cuh"
#undef private

#define main reference_cylinder2d_main
#include "main.cu"
#undef main

namespace {

// Cells sharing at least one vertex with each cell, ascending, the cell itself excluded.
void fill_neighbours(Mesh2D& mesh)
{
    const auto& cells = mesh.getHostCells();
    const int nc = mesh.getCells().size;
    int nv = 0;
    for (int c = 0; c < nc; ++c)
        nv = std::max<int>(nv, std::max(cells[c].x, std::max(cells[c].y, cells[c].z)) + 1);
    std::vector<int> off(nv + 1, 0), inc;
    for (int c = 0; c < nc; ++c) {
        ++off[cells[c].x + 1];
        ++off[cells[c].y + 1];
        ++off[cells[c].z + 1];
    }
    for (int i = 0; i < nv; ++i) off[i + 1] += off[i];
    inc.resize(off[nv]);
    std::vector<int> fill(off.begin(), off.end() - 1);
    for (int c = 0; c < nc; ++c) {
        inc[fill[cells[c].x]++] = c;
        inc[fill[cells[c].y]++] = c;
        inc[fill[cells[c].z]++] = c;
    }
    std::vector<int> nb_off(nc + 1, 0), nb, row;
    nb.reserve((size_t)nc * 13);
    for (int c = 0; c < nc; ++c) {
        row.clear();
        const unsigned v[3] = { cells[c].x, cells[c].y, cells[c].z };
        for (unsigned w : v)
            for (int k = off[w]; k < off[w + 1]; ++k)
                if (inc[k] != c) row.push_back(inc[k]);
        std::sort(row.begin(), row.end());
        row.erase(std::unique(row.begin(), row.end()), row.end());
        nb.insert(nb.end(), row.begin(), row.end());
        nb_off[c + 1] = (int)nb.size();
    }
    mesh.cellNeighborsOffsets.allocate(nc + 1);
    mesh.cellNeighborIndices.allocate((int)nb.size());
    copy_h2d(nb_off.data(), mesh.cellNeighborsOffsets.data, nc + 1);
    copy_h2d(nb.data(), mesh.cellNeighborIndices.data, (int)nb.size());
}

const char* kPhaseNames[8] = { "particles", "projection", "prediction", "pressure_assembly",
                              "pressure_solve", "correction", "particle_correction", "loads" };

}  // namespace

int main(int argc, char* argv[])
{
    if (argc != 9) {
        fprintf(stderr, "usage: %s MESH.dat LEVEL DT SCHEME jacobi|ic WARMUP STEPS OUT.json\n", argv[0]);
        return 2;
    }
    const std::string meshPath = argv[1];
    const int level = atoi(argv[2]);
    const double dt = atof(argv[3]);
    const int scheme = atoi(argv[4]);
    const bool useIC = std::string(argv[5]) == "ic";
    const int warmup = atoi(argv[6]);
    const int steps = atoi(argv[7]);
    const std::string outPath = argv[8];

    Mesh2D mesh;
    if (!mesh.loadMeshFromFile(meshPath, false)) return EXIT_FAILURE;
    fill_neighbours(mesh);
    unsigned int blocks = blocksForSize(mesh.getCells().size);
    kSetEdgeBoundaryIDs<<<blocks, gpuThreads>>>(mesh.getCells().size, mesh.getVertices().data, mesh.getCells().data,
                                                mesh.getEdgeBoundaryIDs().data);

    ParticleHandler2D particleHandler(&mesh, level);
    particleHandler.seedParticles();
    const int problemSize = mesh.getVertices().size;

    // boundary nodes as the case classifies them (main.cu:666-695)
    std::array<DirichletBCs, 2> velocityBCs;
    std::array<VelocityDirichletBCs, 2> velocityPredictionBCs;
    DirichletBCs pressureBCs;
    {
        std::array<std::vector<DirichletNode>, 2> hv;
        std::vector<DirichletNode> hp;
        const auto& vertices = mesh.getHostVertices();
        for (unsigned i = 0; i < vertices.size(); ++i) {
            const Point2& node = vertices[i];
            const bool inflow = std::fabs(node.x) < CONSTANTS::DOUBLE_MIN;
            const bool outflow = !inflow && std::fabs(node.x - l) < CONSTANTS::DOUBLE_MIN;
            const bool wall = !inflow && !outflow &&
                              (std::fabs(node.y) < CONSTANTS::DOUBLE_MIN || std::fabs(node.y - h) < CONSTANTS::DOUBLE_MIN);
            const bool body = !inflow && !outflow && !wall &&
                              std::fabs(GEOMETRY::distance(node, cylinderCenter) - 0.05) < 0.001;
            if (inflow) {
                hv[0].push_back({ i, 4 * 1.5 * node.y * (h - node.y) / (h * h) });
                hv[1].push_back({ i, 0.0 });
            } else if (outflow) {
                hp.push_back({ i, 0.0 });
            } else if (wall || body) {
                hv[0].push_back({ i, 0.0 });
                hv[1].push_back({ i, 0.0 });
            }
        }
        for (int i = 0; i < 2; ++i) {
            velocityBCs[i].setupDirichletBCs(hv[i]);
            velocityPredictionBCs[i].setupDirichletBCs(hv[i]);
            velocityPredictionBCs[i].setMesh(mesh);
            velocityPredictionBCs[i].setupNodeMap(problemSize, hv[i]);
        }
        pressureBCs.setupDirichletBCs(hp);
    }

    const auto faceQ = createFaceQuadratureFormula(1);
    const auto edgeQ = createEdgeQuadratureFormula(1);
    const int nFace = faceQ.size(), nEdge = edgeQ.size();
    copy_h2const(faceQ.data(), faceQuadratureFormula, nFace);
    copy_h2const(&nFace, &faceQuadraturePointsNum, 1);
    copy_h2const(edgeQ.data(), edgeQuadratureFormula, nEdge);
    copy_h2const(&nEdge, &edgeQuadraturePointsNum, 1);

    SimulationParameters hostParams;
    hostParams.setDefaultParameters();
    hostParams.dt = dt;
    hostParams.mu = 0.001;
    hostParams.simulationScheme = scheme;
    hostParams.tFinal = 1e30;
    hostParams.outputFrequency = 1 << 30;
    hostParams.exportParticles = 0;
    hostParams.calculateLoads = 1;
    hostParams.bodyBoundaryID = 3;
    hostParams.thickness = 0.1;
    copy_h2const(&hostParams, &simParams, 1);

    std::array<SparseMatrixCSR, 2> velocityCorrectionMatrix;
    std::array<SparseMatrixCSR, 2> velocityPredictionMatrix;
    SparseMatrixCSR pressureMatrix(mesh);
    std::array<deviceVector<double>, 2> velocitySolution, velocitySolutionOld, velocityPrediction;
    deviceVector<double> pressureSolution, pressureSolutionOld;
    std::array<deviceVector<double>, 2> velocityCorrectionRhs, velocityPredictionRhs;
    deviceVector<double> pressureRhs;
    for (int i = 0; i < 2; ++i) {
        velocityCorrectionMatrix[i].initialize(mesh);
        velocityPredictionMatrix[i].initialize(mesh);
        velocitySolution[i].allocate(problemSize);
        velocitySolutionOld[i].allocate(problemSize);
        velocityPrediction[i].allocate(problemSize);
        velocityCorrectionRhs[i].allocate(problemSize);
        velocityPredictionRhs[i].allocate(problemSize);
    }
    pressureSolution.allocate(problemSize);
    if (scheme == 1) pressureSolutionOld.allocate(problemSize);
    pressureRhs.allocate(problemSize);
    for (int i = 0; i < 2; ++i) {
        velocitySolution[i].clearValues();
        velocityPrediction[i].clearValues();
    }
    pressureSolution.clearValues();
    if (scheme == 1) pressureSolutionOld.clearValues();

    CylinderIntegrator integrator(mesh);
    integrator.setupVelocityPrediction(velocityPredictionMatrix, velocityPredictionRhs, velocityPrediction);
    integrator.setupPressure(pressureMatrix, pressureRhs, pressureSolution, pressureSolutionOld);
    integrator.setupVelocityCorrection(velocityCorrectionMatrix, velocityCorrectionRhs, velocitySolution,
                                       velocitySolutionOld);
    particleHandler.initParticleVelocity(integrator.getVelocitySolution());

    LinearAlgebra LA;
    PreconditionerJacobi precond(problemSize, &LA);
    SolverCG cgSolver(hostParams.tolerance, hostParams.maxIterations, &LA, &precond);
    cgSolver.init(pressureMatrix);
    PreconditionerIC* precondIC = useIC ? new PreconditionerIC(pressureMatrix, &LA) : nullptr;
    SolverCG* pressureIC = useIC ? new SolverCG(hostParams.tolerance, hostParams.maxIterations, &LA, precondIC)
                                 : nullptr;
    if (pressureIC) pressureIC->init(pressureMatrix);
    SolverCG& pressureSolver = pressureIC ? *pressureIC : cgSolver;
    SolverGMRES gmresSolver(hostParams.tolerance, hostParams.maxIterations, &LA, &precond);
    gmresSolver.init(velocityCorrectionMatrix[0]);
    boundaryLoadsCalculator blCalc(mesh, hostParams);

    GpuTimer timer;
    cudaEvent_t ev[6], e[5];
    for (auto& x : ev) cudaEventCreate(&x);
    for (auto& x : e) cudaEventCreate(&x);
    double phaseSum[8] = { 0 };
    std::vector<double> stepMs;
    cudaDeviceSynchronize();
    auto wallTimed = std::chrono::steady_clock::now();
    double t = hostParams.dt;
    timer.start();  // once, as the case does: stop() then gives each step's time
    for (int s = 0; s < warmup + steps; ++s, t += hostParams.dt) {
        if (s == warmup) {
            cudaDeviceSynchronize();
            wallTimed = std::chrono::steady_clock::now();
        }
        printf("\nTime step no. %d, time = %f\n", s + 1, t);
        cudaEventRecord(ev[0]);
        particleHandler.advectParticles(integrator.getVelocitySolution(), hostParams.dt,
                                        hostParams.particleAdvectionSubsteps);
        cudaEventRecord(ev[1]);
        particleHandler.projectVelocityOntoGrid(integrator.getVelocitySolution());
        for (int i = 0; i < 2; ++i) copy_d2d(velocitySolution[i].data, velocitySolutionOld[i].data, problemSize);
        if (scheme == 1) copy_d2d(pressureSolution.data, pressureSolutionOld.data, problemSize);
        cudaEventRecord(ev[2]);
        float pa = 0.f, pp = 0.f, pc = 0.f, ps = 0.f;
        for (int nOuterIter = 0; nOuterIter < 2; ++nOuterIter) {
            cudaEventRecord(e[0]);
            for (int i = 0; i < 2; ++i) {
                velocityPredictionMatrix[i].clearValues();
                velocityPredictionRhs[i].clearValues();
            }
            integrator.assembleVelocityPrediction();
            for (int i = 0; i < 2; ++i) {
                velocityPredictionBCs[i].setDirichletValues(velocityBCs[i], pressureSolution, pressureSolutionOld, i);
                velocityPredictionBCs[i].applyBCs(velocityPredictionMatrix[i], velocityPredictionRhs[i]);
                gmresSolver.solve(velocityPredictionMatrix[i], velocityPrediction[i], velocityPredictionRhs[i]);
            }
            cudaEventRecord(e[1]);
            pressureMatrix.clearValues();
            pressureRhs.clearValues();
            integrator.assemblePressureEquation();
            pressureBCs.applyBCs(pressureMatrix, pressureRhs);
            cudaEventRecord(e[2]);
            pressureSolver.solve(pressureMatrix, pressureSolution, pressureRhs);
            cudaEventRecord(e[3]);
            for (int i = 0; i < 2; ++i) {
                velocityCorrectionMatrix[i].clearValues();
                velocityCorrectionRhs[i].clearValues();
            }
            integrator.assembleVelocityCorrection();
            for (int i = 0; i < 2; ++i) {
                velocityBCs[i].applyBCs(velocityCorrectionMatrix[i], velocityCorrectionRhs[i]);
                cgSolver.solve(velocityCorrectionMatrix[i], velocitySolution[i], velocityCorrectionRhs[i]);
            }
            cudaEventRecord(e[4]);
            cudaEventSynchronize(e[4]);
            float ms;
            cudaEventElapsedTime(&ms, e[0], e[1]); pp += ms;
            cudaEventElapsedTime(&ms, e[1], e[2]); pa += ms;
            cudaEventElapsedTime(&ms, e[2], e[3]); ps += ms;
            cudaEventElapsedTime(&ms, e[3], e[4]); pc += ms;
        }
        cudaEventRecord(ev[3]);
        particleHandler.correctParticleVelocity(integrator.getVelocitySolution(), integrator.getVelocitySolutionOld());
        cudaEventRecord(ev[4]);
        blCalc.calculateLoads(t, integrator.getVelocitySolution(), pressureSolution);
        cudaEventRecord(ev[5]);
        const float2 times = timer.stop();
        printf("Time of a simulation step: %6.3f ms\n", times.x);
        if (s >= warmup) {
            stepMs.push_back(times.x);
            float ms;
            cudaEventElapsedTime(&ms, ev[0], ev[1]); phaseSum[0] += ms;
            cudaEventElapsedTime(&ms, ev[1], ev[2]); phaseSum[1] += ms;
            phaseSum[2] += pp;
            phaseSum[3] += pa;
            phaseSum[4] += ps;
            phaseSum[5] += pc;
            cudaEventElapsedTime(&ms, ev[3], ev[4]); phaseSum[6] += ms;
            cudaEventElapsedTime(&ms, ev[4], ev[5]); phaseSum[7] += ms;
        }
        fflush(stdout);
    }
    cudaDeviceSynchronize();
    const double wallTimedS = std::chrono::duration<double>(std::chrono::steady_clock::now() - wallTimed).count();
    const cudaError_t err = cudaGetLastError();

    std::ofstream out(outPath);
    out << "{\"steps\": " << stepMs.size() << ", \"warmup\": " << warmup << ", \"particles\": "
        << particleHandler.getParticleCount() << ", \"wall_s_timed\": " << wallTimedS << ", \"step_ms\": [";
    for (size_t k = 0; k < stepMs.size(); ++k) out << (k ? ", " : "") << stepMs[k];
    out << "], \"phase_ms\": {";
    for (int k = 0; k < 8; ++k)
        out << (k ? ", " : "") << "\"" << kPhaseNames[k] << "\": " << (stepMs.empty() ? 0.0 : phaseSum[k] / stepMs.size());
    out << "}, \"cuda_error\": \"" << cudaGetErrorString(err) << "\"}\n";
    out.close();
    delete pressureIC;
    delete precondIC;
    return err == cudaSuccess ? EXIT_SUCCESS : EXIT_FAILURE;
}
