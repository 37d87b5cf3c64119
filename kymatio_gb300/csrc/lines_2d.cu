// Line-split variants of the sizes that need more than one CTA's shared
// memory: 256x256 inputs at J=3 (padded 272) and J=4 (padded 288).
#include "lines.cuh"
KYM_LINES_VARIANT(272, 272, 34, 34)
KYM_LINES_FOLD(272, 272, 34, 34, 0)
KYM_LINES_FOLD(272, 272, 34, 34, 1)
KYM_LINES_VARIANT(288, 288, 18, 18)
KYM_LINES_FOLD(288, 288, 18, 18, 0)
KYM_LINES_FOLD(288, 288, 18, 18, 1)
