// stress_mts.cu -- the stress kernel for 12-system crystals with MTS hardening (h_type 2): the
// same translation unit as stress.cu, compiled with the MTS slip-resistance law.
#define CPFFT_NSLIP 12
#define CPFFT_LAW 2
#define CPFFT_STRESS_LAUNCH launch_stress_mts
#include "stress.cu"
