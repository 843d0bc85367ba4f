// les_col_sj128.cu -- the register-column marches compiled for a row stride of
// 128 cells (grids with nz = 128); device code in les_col_march.cuh.
#include "les_col_march.cuh"

LES_COL_STRIDE_UNIT(128)
