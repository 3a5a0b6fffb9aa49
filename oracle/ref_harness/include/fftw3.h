/* Opaque FFTW plan types so that the reference's fft.h compiles without
   FFTW; the reference-side FFT member functions are provided by the
   harness (ref_stubs.cxx) on top of the oracle's halfcomplex transforms. */
#ifndef MHH_REF_FFTW3_STUB_H
#define MHH_REF_FFTW3_STUB_H
typedef struct fftw_plan_s* fftw_plan;
typedef struct fftwf_plan_s* fftwf_plan;
#endif
