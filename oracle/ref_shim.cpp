// ref_shim.cpp -- test infrastructure only (the oracle's checker, never shipped).
//
// Compiles the reference's own integer building blocks straight from the
// reference tree (no copies) and exports them through a C ABI so that tests can
// pin the oracle and the CUDA library against them:
//   include/fluid/curves.h:56-72    zCurveGridIndexAtCoord  (30-bit Morton encode)
//   include/fluid/curves.h:29-54    coordAtZCurveGridIndex0/1/2 (decode)
//   include/fluid/mctable.hpp:7,44,305  EdgeTable / TriTable / NumVertsTable (C++ copy)
//   include/fluid/mc.h:8,44,305         the same tables, OpenCL copy used by the kernels
// Built by oracle/Makefile into oracle/_ref/ only where the reference tree exists.
#include <array>
#include <cstddef>
#include <cstdint>

struct RefUint3 {
    size_t x, y, z;
};
#define CURVE_UINT3_TYPE RefUint3
#define CURVE_UINT3_CTOR(x, y, z) (RefUint3{(x), (y), (z)})
#include "curves.h"
#include "mctable.hpp"

// mc.h is OpenCL C; skip its cl_types.h include and give it the two typedefs
// and the address-space keyword it needs.
#define LIBFLUID_CL_TYPES
typedef unsigned int uint;
typedef unsigned char uchar;
#define constant
#include "mc.h"
#undef constant

extern "C" {
uint64_t ref_morton(uint64_t x, uint64_t y, uint64_t z) {
    return zCurveGridIndexAtCoord((size_t)x, (size_t)y, (size_t)z);
}
uint64_t ref_morton_decode(uint64_t key, int axis) {
    if (axis == 0) return coordAtZCurveGridIndex0((size_t)key);
    if (axis == 1) return coordAtZCurveGridIndex1((size_t)key);
    return coordAtZCurveGridIndex2((size_t)key);
}
int ref_edge_table(int c) { return mctable::EdgeTable[c]; }
int ref_tri_table(int c, int i) { return mctable::TriTable[c][i]; }
int ref_num_verts(int c) { return mctable::NumVertsTable[c]; }
int ref_cl_edge_table(int c) { return (int)EdgeTable[c]; }
int ref_cl_tri_table(int c, int i) { return (int)TriTable[c][i]; }
int ref_cl_num_verts(int c) { return (int)NumVertsTable[c]; }
}
