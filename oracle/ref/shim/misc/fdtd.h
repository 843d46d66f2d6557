/*
 * Test infrastructure (the CPU oracle build only).  src/omd/fdtd.cpp includes
 * <misc/fdtd.h>; the reference ships that header as include/misc/fdtd.hpp.
 */
#include <misc/fdtd.hpp>
