/*
 * minimmerflow_gb300.hpp -- C++ host adapter over the C ABI (mmf_gb300.h)
 * with the reference's entry points and argument meaning:
 *
 *   mmf_gb300::euler::computeRHS            <- euler::computeRHS           (src/euler.hpp:41-43)
 *   mmf_gb300::reconstruction::computePolynomials
 *                                           <- reconstruction::computePolynomials (src/reconstruction.hpp:41-42)
 *   mmf_gb300::utils::conservative2primitive / primitive2conservative
 *                                           <- utils::*                    (src/utils.hpp:34-35)
 *   mmf_gb300::euler::evalSplitting         <- euler::evalSplitting        (src/euler.hpp:37)
 *   mmf_gb300::euler::evalFluxes            <- euler::evalFluxes           (src/euler.hpp:39)
 *   mmf_gb300::euler::evalInterfaceBCValues <- euler::evalInterfaceBCValues (src/euler.hpp:45-48)
 *   mmf_gb300::reconstruction::eval         <- reconstruction::eval        (src/reconstruction.hpp:44)
 *   mmf_gb300::Stepper                      <- the SSP-RK3 loop            (src/main.cpp:377-506)
 *
 * Header-only C++11.  The mesh and storage types are template parameters so
 * the same code binds to bitpit's MeshGeometricalInfo / PiercedStorage in
 * minimmerflow (or to any type with the same methods):
 *   MeshInfo:    getDimension(), getCellRawIds(), rawGetCellCentroid(raw),
 *                rawGetCellSize(raw), rawGetCellVolume(raw), getInterfaceRawIds(),
 *                rawGetInterfaceNormal(raw), rawGetInterfaceArea(raw),
 *                getPatch().getInterfaces().rawAt(raw).{getOwner,getNeigh}(),
 *                getPatch().getCellConstIterator(id).getRawIndex()
 *   Storages:    rawData(raw) (AoS, contiguous over the raw positions), rawAt(raw)
 *
 * Error behaviour follows the reference: unsupported configurations throw
 * std::runtime_error (src/problem.cpp:57); a non-physical state is reported,
 * not fatal (src/euler.cpp:93-101 only logs it).
 */
#ifndef MINIMMERFLOW_GB300_HPP
#define MINIMMERFLOW_GB300_HPP

#include "mmf_gb300.h"

#include <array>
#include <cmath>
#include <cstdint>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace mmf_gb300 {

inline void check(int rc)
{
    if (rc != MMF_OK) throw std::runtime_error(std::string("mmf_gb300: ") + mmf_last_error());
}

/* A context bound to one mesh: the uniform Cartesian grid recognised from the
 * mesh geometry, its border conditions and the raw-id -> grid-cell map. */
class Context {
public:
    Context(const mmf_grid &grid, const std::vector<int64_t> &rawToCell, int device = 0)
    {
        check(mmf_create(&grid, device, &m_ctx));
        m_n = (int64_t)rawToCell.size();
        bool identity = true;
        for (int64_t r = 0; r < m_n && identity; ++r) identity = (rawToCell[r] == r);
        if (!identity) check(mmf_set_cell_map(m_ctx, m_n, rawToCell.data()));
    }
    ~Context() { mmf_destroy(m_ctx); }
    Context(const Context &) = delete;
    Context &operator=(const Context &) = delete;

    mmf_ctx *get() const { return m_ctx; }
    int64_t nCells() const { return m_n; }

private:
    mmf_ctx *m_ctx = nullptr;
    int64_t m_n = 0;
};

/* The primitive state (p, u, v, w, T) behind the Dirichlet border faces of a
 * problem (problem::getBorderBCInfo, src/problem.cpp:446-470): the
 * forward-facing step's Mach 3 inflow; zero for the other problems, which
 * have no Dirichlet faces. */
inline std::array<double, 5> dirichletState(int problemType)
{
    std::array<double, 5> prim = {{0.0, 0.0, 0.0, 0.0, 0.0}};
    if (problemType == MMF_FFSTEP) prim = {{1.0, 3.0, 0.0, 0.0, 1.0 / 1.4}};
    return prim;
}

/* Recognises the uniform Cartesian grid behind a MeshGeometricalInfo (all
 * cells of one size h on a full nx x ny (x nz) lattice) and the border
 * condition of each side from the interface BC storage. */
template <class MeshInfo, class InterfaceStorageInt>
mmf_grid describeGrid(const MeshInfo &meshInfo, const InterfaceStorageInt &interfaceBCs, int order, int arith,
                      std::vector<int64_t> *rawToCell, int problemType = -1)
{
    mmf_grid g;
    g.dim = meshInfo.getDimension();
    g.order = order;
    g.arith = arith;
    g.chunk = 0;
    const std::array<double, 5> dp = dirichletState(problemType);
    for (int k = 0; k < 5; ++k) g.dirichlet_prim[k] = dp[k];
    const std::vector<std::size_t> &cells = meshInfo.getCellRawIds();
    if (cells.empty()) throw std::runtime_error("mmf_gb300: empty mesh");
    double h = meshInfo.rawGetCellSize(cells[0]);
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    std::size_t maxRaw = 0;
    for (std::size_t raw : cells) {
        if (meshInfo.rawGetCellSize(raw) != h) throw std::runtime_error("mmf_gb300: non-uniform mesh");
        const std::array<double, 3> &c = meshInfo.rawGetCellCentroid(raw);
        for (int d = 0; d < 3; ++d) { lo[d] = std::min(lo[d], c[d]); hi[d] = std::max(hi[d], c[d]); }
        maxRaw = std::max(maxRaw, raw);
    }
    g.h = h;
    for (int d = 0; d < 3; ++d) {
        const bool active = d < g.dim;
        g.n[d] = active ? (int)std::llround((hi[d] - lo[d]) / h) + 1 : 1;
        g.origin[d] = active ? lo[d] - 0.5 * h : lo[d];
        g.bc_lo[d] = g.bc_hi[d] = MMF_BC_FREE_FLOW;
    }
    const int64_t nGrid = (int64_t)g.n[0] * g.n[1] * g.n[2];
    if ((int64_t)cells.size() != nGrid || (int64_t)maxRaw + 1 != nGrid)
        throw std::runtime_error("mmf_gb300: the mesh is not a full uniform grid with contiguous raw ids");
    rawToCell->assign((std::size_t)nGrid, -1);
    for (std::size_t raw : cells) {
        const std::array<double, 3> &c = meshInfo.rawGetCellCentroid(raw);
        int64_t idx[3] = {0, 0, 0};
        for (int d = 0; d < g.dim; ++d) idx[d] = std::llround((c[d] - g.origin[d]) / h - 0.5);
        (*rawToCell)[raw] = idx[0] + (int64_t)g.n[0] * (idx[1] + (int64_t)g.n[1] * idx[2]);
    }
    // border conditions: one code per side, read from the border interfaces
    bool seen[2][3] = {{false, false, false}, {false, false, false}};
    for (std::size_t raw : meshInfo.getInterfaceRawIds()) {
        if (meshInfo.getPatch().getInterfaces().rawAt(raw).getNeigh() >= 0) continue;
        const std::array<double, 3> &nrm = meshInfo.rawGetInterfaceNormal(raw);
        int d = 0;
        for (int q = 1; q < 3; ++q) if (std::fabs(nrm[q]) > std::fabs(nrm[d])) d = q;
        const int side = nrm[d] > 0 ? 1 : 0;
        const int bc = (int)interfaceBCs.rawAt(raw);
        int &slot = side ? g.bc_hi[d] : g.bc_lo[d];
        if (seen[side][d] && slot != bc) throw std::runtime_error("mmf_gb300: mixed border conditions on one side");
        slot = bc;
        seen[side][d] = true;
    }
    return g;
}

namespace detail {
template <class Key>
std::map<const void *, std::unique_ptr<Context>> &contexts()
{
    static std::map<const void *, std::unique_ptr<Context>> m;
    return m;
}
}

/* The context of a mesh, created on first use and kept for later calls. */
template <class MeshInfo, class InterfaceStorageInt>
Context &contextFor(const MeshInfo &meshInfo, const InterfaceStorageInt &interfaceBCs, int order,
                    int arith = MMF_ARITH_REFERENCE, int problemType = -1)
{
    auto &m = detail::contexts<MeshInfo>();
    const void *key = &meshInfo;
    auto it = m.find(key);
    if (it == m.end()) {
        std::vector<int64_t> rawToCell;
        mmf_grid g = describeGrid(meshInfo, interfaceBCs, order, arith, &rawToCell, problemType);
        it = m.emplace(key, std::unique_ptr<Context>(new Context(g, rawToCell))).first;
    }
    return *it->second;
}

template <class MeshInfo>
void releaseContext(const MeshInfo &meshInfo)
{
    detail::contexts<MeshInfo>().erase(&meshInfo);
}

/* A face-list context (mmf_umesh) bound to one mesh: any MeshGeometricalInfo
 * -- non-uniform / refined meshes, immersed bodies, per-face border
 * conditions.  Raw ids with holes are kept: the state buffer is indexed by
 * raw position and the holes are unsolved cells without faces. */
class UContext {
public:
    template <class MeshInfo, class CellStorageBool, class InterfaceStorageInt>
    UContext(const MeshInfo &meshInfo, const CellStorageBool &cellSolvedFlag, const InterfaceStorageInt &interfaceBCs,
             int arith, int problemType = -1, int device = 0)
    {
        const std::vector<std::size_t> &cells = meshInfo.getCellRawIds();
        std::size_t n = 0;
        for (std::size_t raw : cells) n = std::max(n, raw + 1);
        std::vector<double> vol(n, 1.0), size(n, std::numeric_limits<double>::max());
        std::vector<unsigned char> solved(n, 0);
        for (std::size_t raw : cells) {
            vol[raw] = meshInfo.rawGetCellVolume(raw);
            size[raw] = meshInfo.rawGetCellSize(raw);
            solved[raw] = cellSolvedFlag.rawAt(raw) ? 1 : 0;
        }
        const std::vector<std::size_t> &faces = meshInfo.getInterfaceRawIds();
        std::vector<int64_t> owner, neigh;
        std::vector<double> area, normal;
        std::vector<int> bc;
        for (std::size_t raw : faces) {   // src/euler.cpp:153-178: the face loop and its id -> raw lookups
            const auto &itf = meshInfo.getPatch().getInterfaces().rawAt(raw);
            owner.push_back((int64_t)meshInfo.getPatch().getCellConstIterator(itf.getOwner()).getRawIndex());
            const long nid = itf.getNeigh();
            neigh.push_back(nid >= 0 ? (int64_t)meshInfo.getPatch().getCellConstIterator(nid).getRawIndex() : -1);
            area.push_back(meshInfo.rawGetInterfaceArea(raw));
            const std::array<double, 3> &nr = meshInfo.rawGetInterfaceNormal(raw);
            normal.insert(normal.end(), nr.begin(), nr.end());
            bc.push_back((int)interfaceBCs.rawAt(raw));
        }
        mmf_umesh_desc d;
        d.dim = meshInfo.getDimension();
        d.n_cells = (int64_t)n;
        d.n_faces = (int64_t)owner.size();
        d.cell_volume = vol.data();
        d.cell_size = size.data();
        d.solved = solved.data();
        d.owner = owner.data();
        d.neigh = neigh.data();
        d.area = area.data();
        d.normal = normal.data();
        d.bc = bc.data();
        const std::array<double, 5> dp = dirichletState(problemType);
        for (int k = 0; k < 5; ++k) d.dirichlet_prim[k] = dp[k];
        d.arith = arith;
        check(mmf_umesh_create(&d, device, &m_u));
        m_n = (int64_t)n;
    }
    ~UContext() { mmf_umesh_destroy(m_u); }
    UContext(const UContext &) = delete;
    UContext &operator=(const UContext &) = delete;
    mmf_umesh *get() const { return m_u; }
    int64_t nCells() const { return m_n; }

private:
    mmf_umesh *m_u = nullptr;
    int64_t m_n = 0;
};

namespace detail {
template <class Key>
std::map<const void *, std::unique_ptr<UContext>> &ucontexts()
{
    static std::map<const void *, std::unique_ptr<UContext>> m;
    return m;
}

/* true when the mesh is a full uniform grid with one border condition per side
 * and every cell is solved: the Cartesian kernels apply */
template <class MeshInfo, class CellStorageBool, class InterfaceStorageInt>
bool cartesian_applies(const MeshInfo &meshInfo, const CellStorageBool &cellSolvedFlag,
                       const InterfaceStorageInt &interfaceBCs)
{
    for (std::size_t raw : meshInfo.getCellRawIds())
        if (!cellSolvedFlag.rawAt(raw)) return false;
    try {
        std::vector<int64_t> map;
        describeGrid(meshInfo, interfaceBCs, 1, MMF_ARITH_REFERENCE, &map);
    } catch (const std::runtime_error &) {
        return false;
    }
    return true;
}
}

template <class MeshInfo>
void releaseContexts(const MeshInfo &meshInfo)
{
    detail::contexts<MeshInfo>().erase(&meshInfo);
    detail::ucontexts<MeshInfo>().erase(&meshInfo);
}

namespace reconstruction {
/* reconstruction::eval (src/reconstruction.cpp:67-79): the reconstructed
 * state at a point of a cell.  Order 1 is the cell mean (eval_1,
 * src/reconstruction.cpp:89-97); the reference stops for any other order, and
 * so does this host helper (order 2 lives in the device kernels). */
template <class MeshInfo>
void eval(std::size_t, const MeshInfo &, int order, const std::array<double, 3> &, const double *means, double *values)
{
    if (order != 1) throw std::runtime_error("mmf_gb300: reconstruction::eval supports order 1");
    for (int k = 0; k < 5; ++k) values[k] = means[k];
}

/* reconstruction::computePolynomials (src/reconstruction.cpp:47-55): order 1
 * needs no polynomial data. */
template <class ProblemType, class MeshInfo, class CellStorageBool, class CellStorageDouble, class InterfaceStorageInt>
void computePolynomials(ProblemType, const MeshInfo &, const CellStorageBool &, const CellStorageDouble &,
                        const InterfaceStorageInt &)
{
    // order 1: nothing to compute, and no context is created here (the first
    // computeRHS call chooses the Cartesian or the face-list kernels)
}
}

namespace euler {
/* euler::computeRHS (src/euler.cpp:127-249): residual (not divided by the
 * volume) of every cell of 'cellConservatives' into 'cellsRHS', and the
 * maximum face eigenvalue.  A full uniform grid with every cell solved runs
 * on the Cartesian kernels; any other mesh (refined, immersed bodies, per-face
 * border conditions) on the face-list kernels.  Both use the reference
 * arithmetic: the result equals the reference's bit for bit. */
template <class ProblemType, class MeshInfo, class CellStorageBool, class CellStorageDouble, class InterfaceStorageInt>
void computeRHS(ProblemType problemType, const MeshInfo &meshInfo, const CellStorageBool &cellSolvedFlag, int order,
                const CellStorageDouble &cellConservatives, const InterfaceStorageInt &interfaceBCs,
                CellStorageDouble *cellsRHS, double *maxEig)
{
    if (order != 1) throw std::runtime_error("mmf_gb300: only order 1 is supported by this entry point");
    auto &um = detail::ucontexts<MeshInfo>();
    auto uit = um.find(&meshInfo);
    if (uit == um.end() && detail::contexts<MeshInfo>().count(&meshInfo) == 0 &&
        !detail::cartesian_applies(meshInfo, cellSolvedFlag, interfaceBCs))
        uit = um.emplace(&meshInfo, std::unique_ptr<UContext>(new UContext(meshInfo, cellSolvedFlag, interfaceBCs,
                                                                           MMF_ARITH_REFERENCE, (int)problemType)))
                  .first;
    if (uit != um.end()) {
        check(mmf_umesh_compute_rhs(uit->second->get(), cellConservatives.rawData(0), cellsRHS->rawData(0), maxEig,
                                    uit->second->nCells()));
        return;
    }
    Context &ctx = contextFor(meshInfo, interfaceBCs, order, MMF_ARITH_REFERENCE, (int)problemType);
    check(mmf_compute_rhs(ctx.get(), cellConservatives.rawData(0), cellsRHS->rawData(0), maxEig, ctx.nCells()));
}

/* euler::evalSplitting (src/euler.cpp:42-73) for one face. */
inline void evalSplitting(const double *conservativeL, const double *conservativeR, const std::array<double, 3> &n,
                          std::array<double, 5> *fluxes, double *lambda)
{
    check(mmf_eval_splitting(1, conservativeL, conservativeR, n.data(), fluxes->data(), lambda));
}

/* euler::evalFluxes (src/euler.cpp:83-113): the physical flux along n. */
inline void evalFluxes(const double *conservative, const double *primitive, const std::array<double, 3> &n,
                       std::array<double, 5> *fluxes)
{
    check(mmf_eval_fluxes(1, conservative, primitive, n.data(), fluxes->data()));
}

/* euler::evalInterfaceBCValues (src/euler.cpp:261-308): the ghost state
 * behind a border face of the given condition (the point is not used by any
 * condition of the reference; Dirichlet takes the problem's inflow state). */
template <class ProblemType>
void evalInterfaceBCValues(ProblemType problemType, int BCType, const std::array<double, 3> &,
                           const std::array<double, 3> &normal, const double *conservative, double *conservative_BC)
{
    const std::array<double, 5> dp = dirichletState((int)problemType);
    check(mmf_eval_bc_values(1, BCType, normal.data(), conservative, dp.data(), conservative_BC));
}
}

namespace utils {
/* utils::conservative2primitive / primitive2conservative (src/utils.cpp:48-83) */
inline void conservative2primitive(const double *c, double *p) { check(mmf_cons2prim(1, c, p)); }
inline void primitive2conservative(const double *p, double *c) { check(mmf_prim2cons(1, p, c)); }
}

/* The SSP-RK3 loop of src/main.cpp:377-506 kept on the device: upload the
 * state once, advance, download when the host needs it.  A full uniform grid
 * with every cell solved runs on the Cartesian kernels; with the solved flags
 * given, any other mesh (immersed bodies, refined meshes, mixed border
 * conditions) runs on the face-list kernels, unsolved cells keeping their
 * state as in the reference. */
class Stepper {
public:
    template <class MeshInfo, class InterfaceStorageInt>
    Stepper(const MeshInfo &meshInfo, const InterfaceStorageInt &interfaceBCs, int arith = MMF_ARITH_FAST,
            int problemType = -1)
    {
        std::vector<int64_t> rawToCell;
        mmf_grid g = describeGrid(meshInfo, interfaceBCs, 1, arith, &rawToCell, problemType);
        m_ctx.reset(new Context(g, rawToCell));
    }
    template <class MeshInfo, class CellStorageBool, class InterfaceStorageInt>
    Stepper(const MeshInfo &meshInfo, const CellStorageBool &cellSolvedFlag, const InterfaceStorageInt &interfaceBCs,
            int arith, int problemType)
    {
        if (detail::cartesian_applies(meshInfo, cellSolvedFlag, interfaceBCs)) {
            std::vector<int64_t> rawToCell;
            mmf_grid g = describeGrid(meshInfo, interfaceBCs, 1, arith, &rawToCell, problemType);
            m_ctx.reset(new Context(g, rawToCell));
        } else {
            m_uctx.reset(new UContext(meshInfo, cellSolvedFlag, interfaceBCs, arith, problemType));
        }
    }
    /* true when the face-list kernels run this mesh */
    bool faceList() const { return m_uctx != nullptr; }
    template <class CellStorageDouble>
    void upload(const CellStorageDouble &U)
    {
        if (m_uctx) check(mmf_umesh_upload(m_uctx->get(), U.rawData(0), m_uctx->nCells()));
        else check(mmf_upload_state(m_ctx->get(), U.rawData(0), m_ctx->nCells()));
    }
    template <class CellStorageDouble>
    void download(CellStorageDouble *U)
    {
        if (m_uctx) check(mmf_umesh_download(m_uctx->get(), U->rawData(0), m_uctx->nCells()));
        else check(mmf_download_state(m_ctx->get(), U->rawData(0), m_ctx->nCells()));
    }
    void setTime(double cfl, double t, double tMax, int64_t maxSteps = -1)
    {
        if (m_uctx) check(mmf_umesh_time_setup(m_uctx->get(), cfl, t, tMax, maxSteps));
        else check(mmf_time_setup(m_ctx->get(), cfl, t, tMax, maxSteps));
    }
    /* runs until tMax (or maxSteps); returns the number of steps */
    int64_t run(double *t, int64_t batch = 4096)
    {
        int64_t total = 0, done = 0;
        do {
            if (m_uctx) check(mmf_umesh_advance(m_uctx->get(), batch, t, &done));
            else check(mmf_advance(m_ctx->get(), batch, t, &done));
            total += done;
        } while (done == batch);
        return total;
    }

private:
    std::unique_ptr<Context> m_ctx;
    std::unique_ptr<UContext> m_uctx;
};

} // namespace mmf_gb300

#endif
