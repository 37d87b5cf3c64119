// Tensor-core variants of the childless cascade tasks: 256x256 at J=3
// (work 136/68, output 32x32), 32/64/128 inputs with a 10x10 low-pass
// (work 80/40/20, output 8x8) and 256x256 at J=4 (work 144/72/36, output 16x16).
#include "tc_cascade.cuh"
KYM_TC_VARIANT(136, 136, 32, 32, 2, 640)
KYM_TC_VARIANT(68, 68, 32, 32, 4, 512)
KYM_TC_VARIANT(68, 68, 32, 32, 2, 512)
KYM_TC_VARIANT(80, 80, 8, 8, 2, 512)
KYM_TC_VARIANT(40, 40, 8, 8, 4, 512)
KYM_TC_VARIANT(40, 40, 8, 8, 2, 512)
KYM_TC_VARIANT(20, 20, 8, 8, 8, 512)
KYM_TC_VARIANT(20, 20, 8, 8, 4, 512)
KYM_TC_VARIANT(20, 20, 8, 8, 2, 512)
KYM_TC_VARIANT(144, 144, 16, 16, 2, 512)
KYM_TC_VARIANT(72, 72, 16, 16, 4, 512)
KYM_TC_VARIANT(72, 72, 16, 16, 2, 512)
KYM_TC_VARIANT(36, 36, 16, 16, 8, 512)
KYM_TC_VARIANT(36, 36, 16, 16, 4, 512)
KYM_TC_VARIANT(36, 36, 16, 16, 2, 512)
