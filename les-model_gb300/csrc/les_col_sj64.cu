// les_col_sj64.cu -- the register-column marches compiled for a row stride of
// 64 cells (grids with nz = 64); device code in les_col_march.cuh.
#include "les_col_march.cuh"

LES_COL_STRIDE_UNIT(64)
