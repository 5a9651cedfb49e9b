/*
 * Driver for the reference numerics compiled against the bitpit stand-in
 * (TEST INFRASTRUCTURE: builds oracle/_ref/mmf_ref, the checker of the C
 * oracle).  It restates the setup and the SSP-RK3 loop of the reference
 * src/main.cpp:197-506 and the error check of src/main.cpp:550-572 without
 * VTK output and MPI; all physics calls go to the reference's own
 * reconstruction::, euler:: and problem:: functions.
 *
 * usage: mmf_ref <problem> <dim> <nCells> <order> <CFL> <t_end|-|inf> [max_steps] [dump.bin]
 *   '-' takes the problem's default end time (problem.cpp:175-211); 'inf'
 *   runs exactly max_steps steps.
 * prints "Final error:  %.12e", the step count and the loop time.
 */
#include "constants.hpp"
#include "euler.hpp"
#include "mesh_info.hpp"
#include "problem.hpp"
#include "reconstruction.hpp"
#include "storage.hpp"
#include "utils.hpp"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>

using namespace bitpit;

namespace bitpit { namespace config { Config root; } }

int main(int argc, char *argv[])
{
    if (argc < 7) {
        std::fprintf(stderr, "usage: %s <problem> <dim> <nCells> <order> <CFL> <t_end|-> [max_steps] [dump]\n", argv[0]);
        return 2;
    }
    config::root["problem"].set("type", argv[1]);
    config::root["problem"].set("dimensions", argv[2]);
    const bool endless = (std::strcmp(argv[6], "inf") == 0);
    if (std::strcmp(argv[6], "-") != 0 && !endless) config::root["problem"]["time"].set("end", argv[6]);
    const int order = std::atoi(argv[4]);
    const double cfl = std::atof(argv[5]);
    const long nCellsPerDirection = std::atol(argv[3]);
    const long maxSteps = (argc > 7) ? std::atol(argv[7]) : -1;
    const char *dump = (argc > 8) ? argv[8] : nullptr;

    const problem::ProblemType problemType = problem::getProblemType();
    int dimensions;
    double length;
    std::array<double, 3> origin;
    problem::getDomainData(problemType, dimensions, &origin, &length);
    const double tMin = problem::getStartTime(problemType, dimensions);
    const double tMax = endless ? std::numeric_limits<double>::infinity()
                                : problem::getEndTime(problemType, dimensions);
    if (endless && maxSteps < 0) {
        std::fprintf(stderr, "'inf' end time needs max_steps\n");
        return 2;
    }

    VolOctree mesh(dimensions, origin, length, length / nCellsPerDirection);
    MeshGeometricalInfo meshInfo(&mesh);
    const std::vector<std::size_t> &cellRawIds = meshInfo.getCellRawIds();
    const std::size_t nCells = cellRawIds.size();
    const std::vector<std::size_t> &internalCellRawIds = meshInfo.getInternalCellRawIds();
    const std::size_t nInternalCells = internalCellRawIds.size();
    const std::vector<std::size_t> &interfaceRawIds = meshInfo.getInterfaceRawIds();
    const std::size_t nInterfaces = interfaceRawIds.size();

    CellStorageBool cellSolvedFlag(1, &mesh.getCells());
    CellStorageDouble cellConservatives(N_FIELDS, &mesh.getCells());
    CellStorageDouble cellConservativesWork(N_FIELDS, &mesh.getCells());
    CellStorageDouble cellRHS(N_FIELDS, &mesh.getCells());
    for (std::size_t i = 0; i < nCells; ++i) cellSolvedFlag.rawSet(cellRawIds[i], true);

    reconstruction::initialize();

    InterfaceStorageInt interfaceBCs(1, &mesh.getInterfaces());
    for (std::size_t i = 0; i < nInterfaces; ++i) {
        const Interface &interface = mesh.getInterfaces().rawAt(interfaceRawIds[i]);
        long interfaceId = interface.getId();
        interfaceBCs[interfaceId] = interface.isBorder() ? problem::getBorderBCType(problemType, interfaceId, meshInfo)
                                                         : BC_NONE;
    }

    for (std::size_t i = 0; i < nCells; ++i) {
        const std::size_t cellRawId = cellRawIds[i];
        const Cell &cell = mesh.getCells().rawAt(cellRawId);
        problem::evalCellInitalConservatives(problemType, cell, meshInfo, cellConservatives.rawData(cellRawId));
    }

    double minCellSize = std::numeric_limits<double>::max();
    for (std::size_t i = 0; i < nInternalCells; ++i)
        minCellSize = std::min(meshInfo.rawGetCellSize(internalCellRawIds[i]), minCellSize);

    auto t0 = std::chrono::steady_clock::now();
    long step = 0;
    double t = tMin;
    while (t < tMax && (maxSteps < 0 || step < maxSteps)) {
        double maxEig;
        reconstruction::computePolynomials(problemType, meshInfo, cellSolvedFlag, cellConservatives, interfaceBCs);
        euler::computeRHS(problemType, meshInfo, cellSolvedFlag, order, cellConservatives, interfaceBCs, &cellRHS, &maxEig);
        double dt = 0.9 * cfl * minCellSize / maxEig;
        if (t + dt > tMax) dt = tMax - t;
        for (std::size_t i = 0; i < nInternalCells; ++i) {
            const std::size_t r = internalCellRawIds[i];
            if (!cellSolvedFlag.rawAt(r)) continue;
            const double cellVolume = meshInfo.rawGetCellVolume(r);
            const double *RHS = cellRHS.rawData(r);
            const double *conservative = cellConservatives.rawData(r);
            double *conservativeTmp = cellConservativesWork.rawData(r);
            for (int k = 0; k < N_FIELDS; ++k) conservativeTmp[k] = conservative[k] + dt * RHS[k] / cellVolume;
        }
        reconstruction::computePolynomials(problemType, meshInfo, cellSolvedFlag, cellConservativesWork, interfaceBCs);
        euler::computeRHS(problemType, meshInfo, cellSolvedFlag, order, cellConservativesWork, interfaceBCs, &cellRHS, &maxEig);
        for (std::size_t i = 0; i < nInternalCells; ++i) {
            const std::size_t r = internalCellRawIds[i];
            if (!cellSolvedFlag.rawAt(r)) continue;
            double cellVolume = meshInfo.rawGetCellVolume(r);
            const double *RHS = cellRHS.rawData(r);
            const double *conservative = cellConservatives.rawData(r);
            double *conservativeTmp = cellConservativesWork.rawData(r);
            for (int k = 0; k < N_FIELDS; ++k)
                conservativeTmp[k] = 0.75 * conservative[k] + 0.25 * (conservativeTmp[k] + dt * RHS[k] / cellVolume);
        }
        reconstruction::computePolynomials(problemType, meshInfo, cellSolvedFlag, cellConservativesWork, interfaceBCs);
        euler::computeRHS(problemType, meshInfo, cellSolvedFlag, order, cellConservativesWork, interfaceBCs, &cellRHS, &maxEig);
        for (std::size_t i = 0; i < nInternalCells; ++i) {
            const std::size_t r = internalCellRawIds[i];
            if (!cellSolvedFlag.rawAt(r)) continue;
            const double cellVolume = meshInfo.rawGetCellVolume(r);
            const double *RHS = cellRHS.rawData(r);
            double *conservative = cellConservatives.rawData(r);
            const double *conservativeTmp = cellConservativesWork.rawData(r);
            for (int k = 0; k < N_FIELDS; ++k)
                conservative[k] = (1. / 3) * conservative[k] + (2. / 3) * (conservativeTmp[k] + dt * RHS[k] / cellVolume);
        }
        t += dt;
        step++;
    }
    auto t1 = std::chrono::steady_clock::now();

    std::array<double, N_FIELDS> evalConservatives;
    double error = 0.;
    for (std::size_t i = 0; i < nInternalCells; ++i) {
        const std::size_t r = internalCellRawIds[i];
        const Cell &cell = mesh.getCells().rawAt(r);
        const long cellId = cell.getId();
        const double *conservatives = cellConservatives.data(cellId);
        problem::evalCellExactConservatives(problemType, cell, meshInfo, t, evalConservatives.data());
        error += std::abs(conservatives[FID_P] - evalConservatives[FID_P]) * meshInfo.getCellVolume(cellId);
    }
    std::printf(" Final error:  %.12e\n", error);
    std::printf(" Steps:  %ld\n", step);
    std::printf(" Final time:  %.17g\n", t);
    std::printf(" Loop seconds:  %.6f\n", std::chrono::duration<double>(t1 - t0).count());
    if (dump) {
        FILE *fp = std::fopen(dump, "wb");
        if (!fp) return 3;
        std::fwrite(cellConservatives.rawData(0), sizeof(double), nCells * N_FIELDS, fp);
        std::fclose(fp);
    }
    return 0;
}
