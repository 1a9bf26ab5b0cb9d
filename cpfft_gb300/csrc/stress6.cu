// stress6.cu -- the stress-update kernel for 6 slip systems (slip_type hcp6, and hcp18,
// whose twelve other systems the reference leaves as zero vectors; src/mod_crystals.f:
// 1208-1759): stress.cu compiled with CPFFT_NSLIP 6.
#define CPFFT_NSLIP 6
#define CPFFT_STRESS_LAUNCH launch_stress6
#include "stress.cu"
