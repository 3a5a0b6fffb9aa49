/* orc_fft.h -- real halfcomplex FFTs for the CPU oracle (TEST INFRASTRUCTURE
   ONLY).  FFTW R2HC / HC2R conventions, unnormalised; element j of sequence s
   is data[s*dist + j*stride]. */
#ifndef ORC_FFT_H
#define ORC_FFT_H
#ifdef __cplusplus
extern "C" {
#endif
void orcfft_r2hc(int n, int howmany, double* data, long stride, long dist);
void orcfft_hc2r(int n, int howmany, double* data, long stride, long dist);
#ifdef __cplusplus
}
#endif
#endif
