/* Minimal stand-in for bitpit's VolOctree header (see bitpit_containers.hpp). */
#ifndef MMF_SHIM_BITPIT_VOLOCTREE_HPP
#define MMF_SHIM_BITPIT_VOLOCTREE_HPP
#include "bitpit_patchkernel.hpp"
namespace bitpit {
typedef VolumeKernel VolOctree;
}
#endif
