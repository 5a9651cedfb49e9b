/* bitpit stand-in (TEST INFRASTRUCTURE): the configuration tree and the
 * standard streams body.cpp reads through bitpit's IO header. */
#ifndef MMF_REF_SHIM_BITPIT_IO_HPP
#define MMF_REF_SHIM_BITPIT_IO_HPP

#include <iostream>
#include <stdexcept>

#include "bitpit_containers.hpp"

#endif
