/* Build shim for compiling the reference's derivative sources standalone:
 * QuadGrav/include/derivs.h includes "TreeNode.h" only for the octant
 * direction constants, which live in include/dendro.h. */
#pragma once
#include "dendro.h"
