// Scalar functions of the imaginary eigenvalues i*mu of a skew matrix for the
// matrix functions of exp.jl: f(i mu) = a(mu) + i b(mu), the result being
// V diag(f(i mu)) V^H (real for a real skew matrix: Re(V f V^H)).
//   exp:  e^{i mu} = cos mu + i sin mu       cos:  cos(i mu) = cosh mu
//   sin:  i sinh mu                          cosh: cosh(i mu) = cos mu
//   sinh: i sin mu                           tan:  i tanh mu
//   tanh: i tan mu                           cot:  -i coth mu
//   coth: -i cot mu                          log:  ln|mu| + i (pi/2) sign(mu)
// cot, coth and log have no value at mu = 0 (the reference throws there):
// *singular is set and the entry is left infinite.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#include "../../include/skewgpu.h"

namespace skew {

__device__ __forceinline__ void skew_scalar_func(int f, double mu, double* a, double* b, bool* singular) {
  switch (f) {
    case SKEW_FUNC_EXP: {
      double s, c;
      sincos(mu, &s, &c);
      *a = c;
      *b = s;
      break;
    }
    case SKEW_FUNC_COS: *a = cosh(mu); *b = 0.0; break;
    case SKEW_FUNC_SIN: *a = 0.0; *b = sinh(mu); break;
    case SKEW_FUNC_COSH: *a = cos(mu); *b = 0.0; break;
    case SKEW_FUNC_SINH: *a = 0.0; *b = sin(mu); break;
    case SKEW_FUNC_TAN: *a = 0.0; *b = tanh(mu); break;
    case SKEW_FUNC_TANH: *a = 0.0; *b = tan(mu); break;
    case SKEW_FUNC_COT:
      *a = 0.0;
      if (mu == 0.0) { *singular = true; *b = -INFINITY; } else { *b = -1.0 / tanh(mu); }
      break;
    case SKEW_FUNC_COTH:
      *a = 0.0;
      if (mu == 0.0) { *singular = true; *b = -INFINITY; } else { *b = -1.0 / tan(mu); }
      break;
    case SKEW_FUNC_LOG:
      if (mu == 0.0) { *singular = true; *a = -INFINITY; *b = 0.0; }
      else { *a = log(fabs(mu)); *b = (mu > 0.0 ? 1.0 : -1.0) * 1.5707963267948966; }
      break;
    default: *a = 0.0; *b = 0.0; *singular = true; break;
  }
}

// symmetry of the result: +1 Hermitian (cos, cosh), -1 skew (sin, sinh, tan, tanh, cot, coth), 0 none
__host__ __device__ inline int skew_func_symmetry(int f) {
  switch (f) {
    case SKEW_FUNC_COS:
    case SKEW_FUNC_COSH: return 1;
    case SKEW_FUNC_SIN:
    case SKEW_FUNC_SINH:
    case SKEW_FUNC_TAN:
    case SKEW_FUNC_TANH:
    case SKEW_FUNC_COT:
    case SKEW_FUNC_COTH: return -1;
    default: return 0;
  }
}

}  // namespace skew
