// Empty stand-in: the hot-path reference sources include the HDF5 C++ header
// only transitively (through hdf5_diagnostics.hpp) and call nothing from it.
#pragma once
