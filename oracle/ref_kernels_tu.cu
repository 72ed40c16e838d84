// Translation unit that compiles the reference's CUDA kernels, unmodified,
// into a cubin for the oracle (test infrastructure only; never shipped).
// Including block_QR.h pulls in TallShinnyQR.h and kernelQR.h, whose explicit
// instantiations emit tsqr_kernel<T>, tsgemm_tsqr<T> and gemm_blockqr<T> for
// float and double.  The include path is the reference checkout, given on
// the nvcc command line by oracle/build_oracle.py.
#include "block_QR.h"
