// stress_ornl.cu -- the stress kernel for 12-system crystals with ORNL hardening (h_type 4,
// twelve dislocation densities): the same translation unit as stress.cu, compiled with
// the dislocation-density solve of mrr.cuh and ORNL's slip law.
#define CPFFT_NSLIP 12
#define CPFFT_LAW 4
#define CPFFT_STRESS_LAUNCH launch_stress_ornl
#include "stress.cu"
