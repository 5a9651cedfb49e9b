/*
 * Driver for the reference numerics compiled against the bitpit stand-in
 * (TEST INFRASTRUCTURE: builds oracle/_ref/mmf_ref, against which the C
 * oracle is compared).  It restates the setup and the SSP-RK3 loop of the reference
 * src/main.cpp:197-506 and the error check of src/main.cpp:550-572 without
 * VTK output and MPI; all physics calls go to the reference's own
 * reconstruction::, euler:: and problem:: functions.
 *
 * usage: mmf_ref <problem> <dim> <nCells> <order> <CFL> <t_end|-|inf> [max_steps] [dump.bin]
 *               [length=L] [body=xmin,ymin,zmin,xmax,ymax,zmax ...] [init=initial.bin]
 *   '-' takes the problem's default end time (problem.cpp:175-211); 'inf'
 *   runs exactly max_steps steps.  length= sets problem.domain.length (the
 *   forward-facing step has no default); each body= adds a box body to the
 *   configuration read by the reference's body::initialize (body.cpp:49-72),
 *   and the fluid / solved flags and the wall faces between fluid and solid
 *   cells are set up as src/main.cpp:222-277 does.
 * prints "Final error:  %.12e", the step count and the loop time.
 */
#include "body.hpp"
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
    // positional [max_steps] [dump], then key=value options
    std::vector<const char *> positional;
    int nBodies = 0;
    const char *initDump = nullptr;
    for (int a = 7; a < argc; ++a) {
        const char *eq = std::strchr(argv[a], '=');
        if (!eq) { positional.push_back(argv[a]); continue; }
        const std::string key(argv[a], eq - argv[a]);
        if (key == "init") {
            initDump = eq + 1;
        } else if (key == "length") {
            config::root["problem"]["domain"].set("length", eq + 1);
        } else if (key == "body") {
            double b[6];
            if (std::sscanf(eq + 1, "%lf,%lf,%lf,%lf,%lf,%lf", &b[0], &b[1], &b[2], &b[3], &b[4], &b[5]) != 6) {
                std::fprintf(stderr, "body=xmin,ymin,zmin,xmax,ymax,zmax\n");
                return 2;
            }
            Config &body = config::root["bodies"]["body" + std::to_string(nBodies++)];
            body.set("type", "box");
            const char *names[6] = {"xMin", "yMin", "zMin", "xMax", "yMax", "zMax"};
            for (int k = 0; k < 6; ++k) {
                char buf[64];
                std::snprintf(buf, sizeof(buf), "%.17g", b[k]);
                body.set(names[k], buf);
            }
        } else {
            std::fprintf(stderr, "unknown option %s\n", argv[a]);
            return 2;
        }
    }
    const long maxSteps = (positional.size() > 0) ? std::atol(positional[0]) : -1;
    const char *dump = (positional.size() > 1) ? positional[1] : nullptr;

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

    body::initialize();

    CellStorageBool cellSolvedFlag(1, &mesh.getCells());
    CellStorageBool cellFluidFlag(1, &mesh.getCells());
    CellStorageDouble cellConservatives(N_FIELDS, &mesh.getCells());
    CellStorageDouble cellConservativesWork(N_FIELDS, &mesh.getCells());
    CellStorageDouble cellRHS(N_FIELDS, &mesh.getCells());
    for (std::size_t i = 0; i < nCells; ++i) {
        const bool isFluid = body::isPointFluid(meshInfo.rawGetCellCentroid(cellRawIds[i]));
        cellFluidFlag.rawSet(cellRawIds[i], isFluid);
        cellSolvedFlag.rawSet(cellRawIds[i], isFluid);
    }

    reconstruction::initialize();

    InterfaceStorageInt interfaceBCs(1, &mesh.getInterfaces());
    for (std::size_t i = 0; i < nInterfaces; ++i) {
        const Interface &interface = mesh.getInterfaces().rawAt(interfaceRawIds[i]);
        long interfaceId = interface.getId();
        if (interface.isBorder()) {
            interfaceBCs[interfaceId] = problem::getBorderBCType(problemType, interfaceId, meshInfo);
        } else {
            const std::size_t ownerRaw = mesh.getCellConstIterator(interface.getOwner()).getRawIndex();
            const std::size_t neighRaw = mesh.getCellConstIterator(interface.getNeigh()).getRawIndex();
            const bool wall = cellFluidFlag.rawAt(ownerRaw) != cellFluidFlag.rawAt(neighRaw);
            interfaceBCs[interfaceId] = wall ? BC_WALL : BC_NONE;
        }
    }

    for (std::size_t i = 0; i < nCells; ++i) {
        const std::size_t cellRawId = cellRawIds[i];
        const Cell &cell = mesh.getCells().rawAt(cellRawId);
        problem::evalCellInitalConservatives(problemType, cell, meshInfo, cellConservatives.rawData(cellRawId));
    }

    if (initDump) {
        FILE *fp = std::fopen(initDump, "wb");
        if (!fp) return 3;
        std::fwrite(cellConservatives.rawData(0), sizeof(double), nCells * N_FIELDS, fp);
        std::fclose(fp);
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
