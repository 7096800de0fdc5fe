/* Exposes the reference's own TensorMult_Hex_nounroll (src/jacobi/impls/tensor/inlinetmulthex.h)
 * under a callable name for the oracle/_ref library. Test infrastructure only: compiled against the
 * reference source tree by oracle/Makefile, never shipped. */
#include "inlinetmulthex.h"
int ref_tensor_mult_hex(int D, const int P[3], const int Q[3], const double *A[3], const double *in, double *out, int imode)
{
  return TensorMult_Hex_nounroll(D, P, Q, A, in, out, (InsertMode)imode);
}
