/* Test infrastructure (oracle): the time step never calls HDF5; the reference's
 * setup.hpp includes this header, so an empty stand-in is enough. */
#pragma once
