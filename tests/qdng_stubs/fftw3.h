// Declarations-only stand-in for the FFTW3 types QDng's src/fft/fft.h names
// (module compile check only; the engine has its own FFT).
#pragma once
typedef double fftw_complex[2];
typedef struct fftw_plan_s *fftw_plan;
