// stress1.cu -- the stress-update kernel for one slip system (slip_type single,
// src/mod_crystals.f:594-603): stress.cu compiled with CPFFT_NSLIP 1.
#define CPFFT_NSLIP 1
#define CPFFT_STRESS_LAUNCH launch_stress1
#include "stress.cu"
