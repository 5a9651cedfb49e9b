/* Minimal stand-in for bitpit's patch kernel (see bitpit_containers.hpp). */
#ifndef MMF_SHIM_BITPIT_PATCHKERNEL_HPP
#define MMF_SHIM_BITPIT_PATCHKERNEL_HPP

#include "bitpit_containers.hpp"

namespace bitpit {

class Cell {
public:
    long m_id = -1;
    bool m_interior = true;
    long getId() const { return m_id; }
    bool isInterior() const { return m_interior; }
};

class Interface {
public:
    long m_id = -1, m_owner = -1, m_neigh = -1;
    long getId() const { return m_id; }
    long getOwner() const { return m_owner; }
    long getNeigh() const { return m_neigh; }
    bool isBorder() const { return m_neigh < 0; }
};

template <typename T>
class PiercedVector : public PiercedKernelBase {
public:
    std::vector<T> items;
    std::size_t rawCount() const override { return items.size(); }
    const T &rawAt(std::size_t pos) const { return items[pos]; }
    const T &rawFind(std::size_t pos) const { return items[pos]; }
    std::size_t size() const { return items.size(); }
};

template <typename T>
class ItemConstIterator {
public:
    ItemConstIterator(const std::vector<T> *v, std::size_t pos) : m_v(v), m_pos(pos) {}
    long getId() const { return (*m_v)[m_pos].getId(); }
    std::size_t getRawIndex() const { return m_pos; }
    const T *operator->() const { return &(*m_v)[m_pos]; }
    const T &operator*() const { return (*m_v)[m_pos]; }
    ItemConstIterator &operator++() { ++m_pos; return *this; }
    bool operator!=(const ItemConstIterator &o) const { return m_pos != o.m_pos; }
private:
    const std::vector<T> *m_v;
    std::size_t m_pos;
};

/* PatchKernel / VolumeKernel: uniform Cartesian grid as VolOctree builds it
 * with uniform refinement.  Cells are row-major (x fastest); interfaces are
 * listed x-faces, then y-faces, then z-faces, each block in (k, j, i) face
 * order; the owner is the lower cell and a border face is owned by the
 * interior cell with the outward normal. */
class PatchKernel {
public:
    typedef ItemConstIterator<Cell> CellConstIterator;
    typedef ItemConstIterator<Interface> InterfaceConstIterator;

    virtual ~PatchKernel() = default;

    int getDimension() const { return m_dim; }
    const PiercedVector<Cell> &getCells() const { return m_cells; }
    const PiercedVector<Interface> &getInterfaces() const { return m_interfaces; }
    long getCellCount() const { return (long)m_cells.size(); }
    long getInternalCellCount() const { return (long)m_cells.size(); }
    long getInterfaceCount() const { return (long)m_interfaces.size(); }
    CellConstIterator getCellConstIterator(long id) const { return CellConstIterator(&m_cells.items, (std::size_t)id); }
    CellConstIterator cellConstBegin() const { return CellConstIterator(&m_cells.items, 0); }
    CellConstIterator cellConstEnd() const { return CellConstIterator(&m_cells.items, m_cells.size()); }
    InterfaceConstIterator interfaceConstBegin() const { return InterfaceConstIterator(&m_interfaces.items, 0); }
    InterfaceConstIterator interfaceConstEnd() const { return InterfaceConstIterator(&m_interfaces.items, m_interfaces.size()); }

protected:
    int m_dim = 2;
    PiercedVector<Cell> m_cells;
    PiercedVector<Interface> m_interfaces;
};

class VolumeKernel : public PatchKernel {
public:
    VolumeKernel(int dim, const std::array<double, 3> &origin, double length, double dh)
    {
        m_dim = dim;
        m_origin = origin;
        m_n = (long)std::llround(length / dh);
        m_h = length / (double)m_n;
        const long nx = m_n, ny = m_n, nz = (dim == 3) ? m_n : 1;
        m_nz = nz;
        m_cells.items.resize(nx * ny * nz);
        for (long g = 0; g < nx * ny * nz; ++g) m_cells.items[g].m_id = g;
        long f = 0;
        for (int d = 0; d < dim; ++d) {
            long cnt[3] = {nx, ny, nz};
            cnt[d] += 1;
            for (long k = 0; k < cnt[2]; ++k)
                for (long j = 0; j < cnt[1]; ++j)
                    for (long i = 0; i < cnt[0]; ++i, ++f) {
                        long idx[3] = {i, j, k};
                        long lo[3] = {i, j, k}, hi[3] = {i, j, k};
                        lo[d] -= 1;
                        Interface itf;
                        itf.m_id = f;
                        FaceGeom g;
                        g.dir = d;
                        g.sign = 1.0;
                        g.pos[0] = origin[0] + ((double)i + 0.5) * m_h;
                        g.pos[1] = origin[1] + ((double)j + 0.5) * m_h;
                        g.pos[2] = (dim == 3) ? origin[2] + ((double)k + 0.5) * m_h : origin[2];
                        g.pos[d] = origin[d] + (double)idx[d] * m_h;
                        if (idx[d] == 0) {
                            itf.m_owner = hi[0] + nx * (hi[1] + ny * hi[2]);
                            g.sign = -1.0;
                        } else if (idx[d] == (d == 0 ? nx : d == 1 ? ny : nz)) {
                            itf.m_owner = lo[0] + nx * (lo[1] + ny * lo[2]);
                        } else {
                            itf.m_owner = lo[0] + nx * (lo[1] + ny * lo[2]);
                            itf.m_neigh = hi[0] + nx * (hi[1] + ny * hi[2]);
                        }
                        m_interfaces.items.push_back(itf);
                        m_faces.push_back(g);
                    }
        }
    }
    double evalCellVolume(long) const { return (m_dim == 3) ? m_h * m_h * m_h : m_h * m_h; }
    double evalCellSize(long) const { return m_h; }
    std::array<double, 3> evalCellCentroid(long id) const
    {
        long i = id % m_n, j = (id / m_n) % m_n, k = id / (m_n * m_n);
        std::array<double, 3> c;
        c[0] = m_origin[0] + ((double)i + 0.5) * m_h;
        c[1] = m_origin[1] + ((double)j + 0.5) * m_h;
        c[2] = (m_dim == 3) ? m_origin[2] + ((double)k + 0.5) * m_h : m_origin[2];
        return c;
    }
    double evalInterfaceArea(long) const { return (m_dim == 3) ? m_h * m_h : m_h; }
    std::array<double, 3> evalInterfaceCentroid(long id) const
    {
        const FaceGeom &g = m_faces[id];
        return {{g.pos[0], g.pos[1], g.pos[2]}};
    }
    std::array<double, 3> evalInterfaceNormal(long id) const
    {
        std::array<double, 3> n = {{0.0, 0.0, 0.0}};
        n[m_faces[id].dir] = m_faces[id].sign;
        return n;
    }
    long cellsPerDirection() const { return m_n; }

private:
    struct FaceGeom { int dir; double sign; double pos[3]; };
    std::array<double, 3> m_origin;
    long m_n = 0, m_nz = 1;
    double m_h = 0.0;
    std::vector<FaceGeom> m_faces;
};

class PatchInfo {
public:
    explicit PatchInfo(PatchKernel const *patch) : m_patch(patch) {}
    virtual ~PatchInfo() = default;
    void setPatch(PatchKernel const *patch) { m_patch = patch; }
    void extract() { _reset(); _extract(); }
protected:
    PatchKernel const *m_patch;
    virtual void _init() = 0;
    virtual void _reset() = 0;
    virtual void _extract() = 0;
};

} // namespace bitpit

#endif
