// Specialised cascade variants: padded sizes 160/80/40/20 with a 10x10
// low-pass (32x32 at J=2, 64x64 at J=3, 128x128 at J=4).
// (padded 160 and 80)
#include "ct_cascade.cuh"
#include "bwd.cuh"
KYM_CT_VARIANT(160, 160, 10, 10, 1, false, 512)
KYM_CT_FOLD(160, 160, 10, 10, 1, false, 512, 0)
KYM_CT_FOLD(160, 160, 10, 10, 1, false, 512, 1)
KYM_CT_VARIANT(80, 80, 10, 10, 1, false, 512)
KYM_CT_FOLD(80, 80, 10, 10, 1, false, 512, 0)
KYM_CT_FOLD(80, 80, 10, 10, 1, false, 512, 1)
KYM_CT_FOLD(80, 80, 10, 10, 1, false, 512, 2)
KYM_BWD_VARIANT(160, 160, 10, 10, 1, false, 512)
KYM_BWD_VARIANT(80, 80, 10, 10, 1, false, 512)
