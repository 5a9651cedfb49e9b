/*
 * Drop-in check of the C++ adapter (include/minimmerflow_gb300.hpp): the
 * reference time loop of src/main.cpp:377-506, written as in the reference,
 * with euler::computeRHS and reconstruction::computePolynomials taken from
 * mmf_gb300::.  Mesh and storage types are the bitpit stand-in of the oracle
 * (test infrastructure); a small MeshGeometricalInfo-like class provides the
 * accessors the adapter reads.  Initial states come from the C oracle.
 *
 * usage: test_dropin <radsod|vortex_xy|ffstep> <dim> <nCells> <steps> <out_loop.bin> <out_stepper.bin> [body]
 * 'body' makes the cells whose centroid lies in [1, 2.5] x [-1.5, 1.5] (x
 * [-10, 10]) solid and their fluid faces walls (main.cpp:222-277); the
 * adapter then runs on the face-list kernels.  'ffstep' is the Mach 3
 * forward-facing step on [0, 3.2]^2: the step [0.6, 4] x [-1, 0.2] is solid,
 * the left border is the Dirichlet inflow, the right one free flow and the
 * others reflecting (problem.cpp:404-432).
 */
#include "bitpit_voloctree.hpp"
#include "minimmerflow_gb300.hpp"
#include "mmf_oracle.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace bitpit { namespace config { Config root; } }
using namespace bitpit;

typedef PiercedStorage<bool, long> CellStorageBool;
typedef PiercedStorage<double, long> CellStorageDouble;
typedef PiercedStorage<int, long> InterfaceStorageInt;

class MeshInfoLike {
public:
    explicit MeshInfoLike(const VolumeKernel &patch) : m_patch(patch)
    {
        for (std::size_t r = 0; r < patch.getCells().size(); ++r) {
            m_cells.push_back(r);
            m_centroids.push_back(patch.evalCellCentroid((long)r));
            m_sizes.push_back(patch.evalCellSize((long)r));
            m_volumes.push_back(patch.evalCellVolume((long)r));
        }
        for (std::size_t r = 0; r < patch.getInterfaces().size(); ++r) {
            m_interfaces.push_back(r);
            m_normals.push_back(patch.evalInterfaceNormal((long)r));
            m_areas.push_back(patch.evalInterfaceArea((long)r));
        }
    }
    int getDimension() const { return m_patch.getDimension(); }
    const VolumeKernel &getPatch() const { return m_patch; }
    const std::vector<std::size_t> &getCellRawIds() const { return m_cells; }
    const std::vector<std::size_t> &getInterfaceRawIds() const { return m_interfaces; }
    const std::array<double, 3> &rawGetCellCentroid(std::size_t r) const { return m_centroids[r]; }
    double rawGetCellSize(std::size_t r) const { return m_sizes[r]; }
    double rawGetCellVolume(std::size_t r) const { return m_volumes[r]; }
    const std::array<double, 3> &rawGetInterfaceNormal(std::size_t r) const { return m_normals[r]; }
    double rawGetInterfaceArea(std::size_t r) const { return m_areas[r]; }

private:
    const VolumeKernel &m_patch;
    std::vector<std::size_t> m_cells, m_interfaces;
    std::vector<std::array<double, 3>> m_centroids, m_normals;
    std::vector<double> m_sizes, m_volumes, m_areas;
};

int main(int argc, char **argv)
{
    if (argc < 7) return 2;
    const int problem = std::strcmp(argv[1], "radsod") == 0   ? ORC_RADSOD
                        : std::strcmp(argv[1], "ffstep") == 0 ? ORC_FFSTEP
                                                              : ORC_VORTEX_XY;
    const int dim = std::atoi(argv[2]);
    const long n = std::atol(argv[3]);
    const int steps = std::atoi(argv[4]);
    std::array<double, 3> origin = (problem == ORC_VORTEX_XY) ? std::array<double, 3>{{-5., -5., -5.}}
                                                              : std::array<double, 3>{{0., 0., 0.}};
    const double length = (problem == ORC_RADSOD) ? 8.0 : (problem == ORC_FFSTEP) ? 3.2 : 10.0;
    const double cfl = 0.45;
    VolOctree mesh(dim, origin, length, length / n);
    MeshInfoLike meshInfo(mesh);
    const std::size_t nCells = meshInfo.getCellRawIds().size();

    CellStorageBool solved(1, &mesh.getCells());
    CellStorageDouble U(5, &mesh.getCells()), W(5, &mesh.getCells()), RHS(5, &mesh.getCells());
    InterfaceStorageInt bcs(1, &mesh.getInterfaces());
    const bool body = argc > 7 && std::strcmp(argv[7], "body") == 0;
    for (std::size_t r = 0; r < nCells; ++r) {
        const std::array<double, 3> &c = meshInfo.rawGetCellCentroid(r);
        bool solid = false;
        if (body && problem == ORC_FFSTEP) solid = c[0] >= 0.6 && c[0] <= 4.0 && c[1] >= -1.0 && c[1] <= 0.2;
        else if (body) solid = c[0] > 1.0 && c[0] < 2.5 && c[1] > -1.5 && c[1] < 1.5;
        solved.rawSet(r, !solid);
    }
    for (std::size_t f : meshInfo.getInterfaceRawIds()) {
        const Interface &itf = mesh.getInterfaces().rawAt(f);
        if (itf.isBorder()) {
            int bc = (problem == ORC_RADSOD ? MMF_BC_REFLECTING : MMF_BC_FREE_FLOW);
            if (problem == ORC_FFSTEP) {
                // problem.cpp:422-432 on the face centroid (owner centroid + h/2 along the normal)
                const double x = meshInfo.rawGetCellCentroid((std::size_t)itf.getOwner())[0] +
                                 0.5 * meshInfo.rawGetCellSize(0) * meshInfo.rawGetInterfaceNormal(f)[0];
                bc = x < 1e-10 ? MMF_BC_DIRICHLET : (x > 3.2 - 1e-10 ? MMF_BC_FREE_FLOW : MMF_BC_REFLECTING);
            }
            bcs[(long)f] = bc;
        } else {
            bcs[(long)f] = (solved.rawAt(itf.getOwner()) != solved.rawAt(itf.getNeigh())) ? MMF_BC_WALL : MMF_BC_NONE;
        }
    }
    // the reference's point-wise entry points through the adapter against the oracle
    {
        const double c[5] = {1.1, 0.3, -0.2, 0.05, 2.7}, nrm3[3] = {0.6, -0.8, 0.0};
        const std::array<double, 3> n3 = {{0.6, -0.8, 0.0}}, pt = {{0.0, 0.0, 0.0}};
        double pr[5], pr_ref[5], f_ref[5], g_ref[5], g[5], v[5];
        mmf_gb300::utils::conservative2primitive(c, pr);
        orc_cons2prim(c, pr_ref);
        std::array<double, 5> f;
        mmf_gb300::euler::evalFluxes(c, pr, n3, &f);
        orc_eval_fluxes(c, pr_ref, nrm3, f_ref);
        for (int k = 0; k < 5; ++k)
            if (pr[k] != pr_ref[k] || f[k] != f_ref[k]) return 4;
        for (int bc : {MMF_BC_FREE_FLOW, MMF_BC_REFLECTING, MMF_BC_WALL, MMF_BC_DIRICHLET}) {
            mmf_gb300::euler::evalInterfaceBCValues(ORC_FFSTEP, bc, pt, n3, c, g);
            orc_eval_bc(ORC_FFSTEP, bc, pt.data(), nrm3, c, g_ref);
            for (int k = 0; k < 5; ++k)
                if (g[k] != g_ref[k]) return 5;
        }
        mmf_gb300::reconstruction::eval(0, meshInfo, 1, pt, c, v);
        for (int k = 0; k < 5; ++k)
            if (v[k] != c[k]) return 6;
    }
    orc_params prm;
    orc_params_default(&prm);
    for (std::size_t r = 0; r < nCells; ++r)
        orc_exact_conservatives(problem, dim, &prm, meshInfo.rawGetCellCentroid(r).data(), 0.0, U.rawData(r));
    CellStorageDouble U0 = U;

    const double minCellSize = meshInfo.rawGetCellSize(0);
    double t = 0.0;
    for (int step = 0; step < steps; ++step) {
        double maxEig;
        mmf_gb300::reconstruction::computePolynomials(problem, meshInfo, solved, U, bcs);
        mmf_gb300::euler::computeRHS(problem, meshInfo, solved, 1, U, bcs, &RHS, &maxEig);
        double dt = 0.9 * cfl * minCellSize / maxEig;
        for (std::size_t r = 0; r < nCells; ++r) {
            if (!solved.rawAt(r)) continue;
            for (int k = 0; k < 5; ++k) W.rawData(r)[k] = U.rawData(r)[k] + dt * RHS.rawData(r)[k] / meshInfo.rawGetCellVolume(r);
        }
        mmf_gb300::euler::computeRHS(problem, meshInfo, solved, 1, W, bcs, &RHS, &maxEig);
        for (std::size_t r = 0; r < nCells; ++r) {
            if (!solved.rawAt(r)) continue;
            for (int k = 0; k < 5; ++k)
                W.rawData(r)[k] = 0.75 * U.rawData(r)[k] + 0.25 * (W.rawData(r)[k] + dt * RHS.rawData(r)[k] / meshInfo.rawGetCellVolume(r));
        }
        mmf_gb300::euler::computeRHS(problem, meshInfo, solved, 1, W, bcs, &RHS, &maxEig);
        for (std::size_t r = 0; r < nCells; ++r) {
            if (!solved.rawAt(r)) continue;
            for (int k = 0; k < 5; ++k)
                U.rawData(r)[k] = (1. / 3) * U.rawData(r)[k] + (2. / 3) * (W.rawData(r)[k] + dt * RHS.rawData(r)[k] / meshInfo.rawGetCellVolume(r));
        }
        t += dt;
    }
    FILE *fp = std::fopen(argv[5], "wb");
    std::fwrite(U.rawData(0), sizeof(double), 5 * nCells, fp);
    std::fclose(fp);

    // the same run kept on the device (face-list kernels when a body is present)
    mmf_gb300::Stepper stepper(meshInfo, solved, bcs, MMF_ARITH_REFERENCE, problem);
    if (stepper.faceList() != body) return 3;
    stepper.upload(U0);
    stepper.setTime(cfl, 0.0, INFINITY, steps);
    double t2 = 0.0;
    const int64_t done = stepper.run(&t2);
    stepper.download(&U0);
    fp = std::fopen(argv[6], "wb");
    std::fwrite(U0.rawData(0), sizeof(double), 5 * nCells, fp);
    std::fclose(fp);
    std::printf("steps %d %lld t %.17g %.17g\n", steps, (long long)done, t, t2);
    mmf_gb300::releaseContexts(meshInfo);
    return (done == steps && t == t2) ? 0 : 1;
}
