// The interior-row table of the host-array pipeline, shared by the device
// side (dgb_api.cu) and the host copies (host_copy.cpp).
#pragma once
#include <stdint.h>

namespace dgb {

// One interior row of a block: padded index relative to its chunk's start,
// position in the chunk's packed interior, length.
struct IRow {
    uint32_t src, dst, len;
};

}  // namespace dgb
