// Shared-fold line-split variants of the childless groups of 256x256 inputs
// at J=3 (padded 272): order 2 (0,1) at 136 from 272 parents, (0,2) at 68
// from 272 parents, (1,2) at 68 from 136 parents (8 x 8 paths each), and
// order 1 j1=2 at 68 from the input spectrum (1 x 8 paths); 34x34 low-pass.
// Template arguments: size, fold, sources, wavelets, low-pass size (rows,
// cols), rows per CTA of the row-FFT pass, columns per CTA of the column
// pass, threads of the rows pass, threads of the column passes.
#include "o2.cuh"
KYM_O2_VARIANT(136, 2, 8, 8, 34, 34, 8, 17, 288, 128)
KYM_O2_VARIANT(68, 4, 8, 8, 34, 34, 34, 17, 256, 128)
KYM_O2_VARIANT(68, 2, 8, 8, 34, 34, 34, 17, 256, 128)
KYM_O2_VARIANT(68, 4, 1, 8, 34, 34, 34, 17, 256, 128)
