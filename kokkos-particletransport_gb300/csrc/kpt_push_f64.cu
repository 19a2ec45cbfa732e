// The plain FP64 interval push (Parker and focused) and the FP64 table
// sampling, emitted from kpt_push.cu into their own translation unit, which
// the build compiles with FMA contraction off (nvcc -fmad=false): every
// double operation rounds as the expression is written, as in the host
// oracle and the reference build (both -ffp-contract=off), so the FP64 push
// follows them bit for bit over whole intervals.  Contraction stays on for
// the mixed-precision kernels in kpt_push.cu.
#define KPT_PUSH_PART 1
#include "kpt_push.cu"
