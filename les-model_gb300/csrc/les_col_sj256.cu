// les_col_sj256.cu -- the register-column marches compiled for a row stride of
// 256 cells (grids with nz = 256); device code in les_col_march.cuh.
#include "les_col_march.cuh"

LES_COL_STRIDE_UNIT(256)
