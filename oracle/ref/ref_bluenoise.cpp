/* ref_bluenoise.cpp - the reference's blue-noise tables (lib/RenderSystem/common_bluenoise.h, Heitz et al.'s
 * published data), compiled by path from the reference tree so that tests can drive the reference's kernels
 * and the oracle with them (TEST INFRASTRUCTURE ONLY; nothing is copied into this repository). The tables are
 * read as bytes, as rendercore_optix7/rendercore.cpp:247-253 does. */
#include <cstdint>
#include "common_bluenoise.h"

extern "C" {
const uint8_t* ref_bluenoise_sobol() { return (const uint8_t*)sob256_64; }
const uint8_t* ref_bluenoise_scrambling() { return (const uint8_t*)scr256_64; }
const uint8_t* ref_bluenoise_ranking() { return (const uint8_t*)rnk256_64; }
}
