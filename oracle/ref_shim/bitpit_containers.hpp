/*
 * Minimal project-written stand-in for the subset of the bitpit library that
 * minimmerflow's src/utils.cpp, src/euler.cpp, src/reconstruction.cpp,
 * src/problem.cpp and src/mesh_info.cpp use.  bitpit is an external
 * dependency that is not vendored with the reference (CMakeLists.txt:103,
 * find_package(BITPIT REQUIRED), version unpinned), so these headers restate
 * only the interfaces those files call: PiercedStorage, VolumeKernel /
 * PatchKernel with a uniform Cartesian "octree", PatchInfo, config, log.
 *
 * TEST INFRASTRUCTURE: used only to compile the reference sources into
 * oracle/_ref, against which the C oracle is compared.
 */
#ifndef MMF_SHIM_BITPIT_CONTAINERS_HPP
#define MMF_SHIM_BITPIT_CONTAINERS_HPP

#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#define BITPIT_UNUSED(x) (void)(x)
#define BITPIT_UNREACHABLE(msg) throw std::runtime_error(msg)

/* element-wise array arithmetic (bitpit's operators.hpp provides these) */
template <typename T, std::size_t N>
std::array<T, N> operator*(const T &s, const std::array<T, N> &a)
{
    std::array<T, N> r;
    for (std::size_t i = 0; i < N; ++i) r[i] = s * a[i];
    return r;
}
template <typename T, std::size_t N>
std::ostream &operator<<(std::ostream &os, const std::array<T, N> &a)
{
    for (std::size_t i = 0; i < N; ++i) os << a[i] << (i + 1 < N ? " " : "");
    return os;
}

namespace bitpit {

class PiercedKernelBase {
public:
    virtual ~PiercedKernelBase() = default;
    virtual std::size_t rawCount() const = 0;
};

/* PiercedStorage: fields stored per raw position; ids equal raw positions here */
template <typename T, typename id_t = long>
class PiercedStorage {
    typedef typename std::conditional<std::is_same<T, bool>::value, unsigned char, T>::type elem_t;
public:
    PiercedStorage() : m_nFields(1), m_kernel(nullptr) {}
    PiercedStorage(std::size_t nFields, const PiercedKernelBase *kernel) : m_nFields(nFields), m_kernel(nullptr)
    {
        setStaticKernel(kernel);
    }
    void setStaticKernel(const PiercedKernelBase *kernel)
    {
        m_kernel = kernel;
        m_data.assign(kernel->rawCount() * m_nFields, elem_t());
    }
    std::size_t getFieldCount() const { return m_nFields; }
    elem_t *rawData(std::size_t pos) { return m_data.data() + pos * m_nFields; }
    const elem_t *rawData(std::size_t pos) const { return m_data.data() + pos * m_nFields; }
    elem_t *data(id_t id) { return rawData((std::size_t)id); }
    const elem_t *data(id_t id) const { return rawData((std::size_t)id); }
    const elem_t &rawAt(std::size_t pos) const { return m_data[pos * m_nFields]; }
    elem_t &rawAt(std::size_t pos) { return m_data[pos * m_nFields]; }
    const elem_t &at(id_t id) const { return m_data[(std::size_t)id * m_nFields]; }
    void rawSet(std::size_t pos, const T &v) { m_data[pos * m_nFields] = v; }
    elem_t &operator[](id_t id) { return m_data[(std::size_t)id * m_nFields]; }
private:
    std::size_t m_nFields;
    const PiercedKernelBase *m_kernel;
    std::vector<elem_t> m_data;
};

namespace log {
inline std::ostream &cout()
{
    static std::ostringstream sink;
    sink.str("");
    return sink;
}
}

class Config {
public:
    Config &operator[](const std::string &key)
    {
        std::unique_ptr<Config> &s = m_sections[key];
        if (!s) s.reset(new Config());
        return *s;
    }
    const Config &operator[](const std::string &key) const
    {
        auto it = m_sections.find(key);
        if (it == m_sections.end()) throw std::runtime_error("missing section " + key);
        return *it->second;
    }
    bool hasSection(const std::string &key) const { return m_sections.count(key) > 0; }
    const std::map<std::string, std::unique_ptr<Config>> &getSections() const { return m_sections; }
    bool hasOption(const std::string &key) const { return m_options.count(key) > 0; }
    void set(const std::string &key, const std::string &value) { m_options[key] = value; }
    template <typename T>
    T get(const std::string &key) const
    {
        auto it = m_options.find(key);
        if (it == m_options.end()) throw std::runtime_error("missing option " + key);
        std::istringstream is(it->second);
        T v;
        is >> v;
        return v;
    }
    template <typename T, typename D>
    T get(const std::string &key, const D &dflt) const
    {
        if (!hasOption(key)) return (T)dflt;
        return get<T>(key);
    }
    void clear() { m_options.clear(); m_sections.clear(); }
private:
    std::map<std::string, std::string> m_options;
    std::map<std::string, std::unique_ptr<Config>> m_sections;
};

namespace config {
extern Config root;
}

} // namespace bitpit

#endif
