// stress_mrr.cu -- the stress kernel for 12-system crystals with Ma-Roters-Raabe hardening
// (h_type 7, twelve dislocation densities): the same translation unit as stress.cu,
// compiled with the MRR law of mrr.cuh.
#define CPFFT_NSLIP 12
#define CPFFT_LAW 7
#define CPFFT_STRESS_LAUNCH launch_stress_mrr
#include "stress.cu"
