// FP64 3-D DFT filter of a prime size by Rader's algorithm (prime_dft.cu).
#pragma once
#include <cufft.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace spf {

struct PrimeDft {
  int p = 0;                            // transform size per axis (prime)
  int nb = 1;                           // independent p^3 arrays in one call
  int64_t lines = 0;                    // nb p^2 lines per axis pass
  int16_t *pinv = nullptr;              // pinv[g^m mod p] = m
  int16_t *qinv = nullptr;              // qinv[g^-q mod p] = q
  double2 *bf = nullptr, *bi = nullptr; // FFT_{p-1}(b) / (p-1), forward / inverse sign
  double2 *a = nullptr;                 // [lines][p-1] Rader-ordered lines
  double2 *x0 = nullptr, *dc = nullptr; // [lines] first element, DC of FFT(a)
  double2 *z = nullptr;                 // [nb][p^3] spectrum between passes
  cufftHandle plan = 0;                 // batched Z2Z of length p-1
  bool plan_ok = false;
};

// p prime, p - 1 a product of 2, 3, 5, 7, 5 <= p <= 32767
bool prime_dft_applies(int p);
int prime_dft_create(int p, int nb, PrimeDft **out);
void prime_dft_free(PrimeDft *d);
// out = Re(IDFT3(h . DFT3(in))) for each of the nb real p^3 arrays, the
// inverse unnormalised (as cuFFT's Z2D); h is a real p^3 multiplier shared
// by the arrays
int prime_dft_filter(PrimeDft *d, const double *in, const double *h, double *out,
                     cudaStream_t s);

}  // namespace spf
