// stress48.cu -- the stress-update kernel for 48 slip systems (slip_type bcc48,
// src/mod_crystals.f:812-1207): stress.cu compiled with CPFFT_NSLIP 48.
#define CPFFT_NSLIP 48
#define CPFFT_STRESS_LAUNCH launch_stress48
#include "stress.cu"
