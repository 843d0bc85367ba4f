// les_col_sj32.cu -- the register-column marches compiled for a row stride of
// 32 cells (grids with nz = 32); device code in les_col_march.cuh.
#include "les_col_march.cuh"

LES_COL_STRIDE_UNIT(32)
