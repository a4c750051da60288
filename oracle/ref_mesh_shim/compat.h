/* Forced-include shim for the oracle build of the reference's octree mesh.
 * Newer libstdc++ rejects abs() of an unsigned int as ambiguous; the
 * reference's sources apply it to differences of unsigned counters in their
 * multi-rank load-balance code.  This overload gives the magnitude of the
 * difference read as a signed int, which is what those call sites mean. */
#pragma once
#include <cstdlib>
static inline long abs(unsigned int x) { return std::labs((long)(int)x); }
