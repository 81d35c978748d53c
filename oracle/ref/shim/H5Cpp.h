// Build-side stand-in for the HDF5 C++ header, which is not installed here:
// src/Saver.h (pulled in by src/Render.h through src/Loader.h) only names
// H5File in declarations, so a forward declaration lets src/Render.cpp
// compile unmodified (with the standard headers the real one includes).
// Nothing in the harness calls the HDF5 functions.
#pragma once
// the real header brings these in; src/Render.cpp relies on them
#include <fstream>
#include <iomanip>
#include <string>
namespace H5 {
class H5File;
}
