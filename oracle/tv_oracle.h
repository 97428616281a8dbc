/* tv_oracle.h -- CPU restatement of the reference decoder (test infrastructure
 * only; see tv_oracle.c).  Plain C ABI so tests load it through ctypes. */
#ifndef TV_ORACLE_H
#define TV_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { TVO_OK = 0, TVO_EINVAL = -1, TVO_ESHORT = -2, TVO_ERANGE = -3, TVO_ENOMEM = -4 };

int tvo_check_args(int N, int O, int D, int T, const int32_t* obs);

void tvo_survival(int N, int D, const double* duration, double* surv);

/* variant 0 = serial (src/hsmm.cu:233-373), 1 = OpenMP (src/hsmm.cu:376-600).
 * Optional outputs (NULL to skip): delta_out (T,N) time-major induction
 * scores, tail_out (N) tail-adjusted scores at T-1, psi_*_out (T,N)
 * back-pointers (row T-1 holds the tail's), seg_start_out (T) 1 where a
 * decoded segment starts. */
int tvo_decode(int N, int O, int D, int T,
               const double* trans, const double* emission,
               const double* start, const double* duration,
               const int32_t* obs, int variant, int nthreads,
               int32_t* path_out, double* loglik_out,
               double* delta_out, double* tail_out,
               int32_t* psi_state_out, int32_t* psi_dur_out,
               uint8_t* seg_start_out);

double tvo_score_segments(int N, int O, int D, int T,
                          const double* trans, const double* emission,
                          const double* start, const double* duration,
                          const int32_t* obs, const int32_t* path,
                          const uint8_t* seg_start);

/* tv_oracle_cuda.c: the reference CUDA backend's values (src/kernels.cu),
 * each of its four differences from the C++ decoder switchable. */
enum { TVO_CU_INIT_SCAN = 1, TVO_CU_WINDOW = 2, TVO_CU_TAIL = 4, TVO_CU_ITREE = 8, TVO_CU_ALL = 15 };
void tvo_block_scan(const double* x, int n, double* out);
void tvo_lin_suffix(int N, int D, const double* dur_lin, double* out);
int tvo_decode_cuda(int N, int O, int D, int T, const double* trans, const double* emission,
                    const double* dur_lin, const double* start, const double* duration,
                    const int32_t* obs, int flags, const double* log_suffix, int nthreads,
                    int32_t* path, double* loglik, double* final);

/* tv_fb_oracle.c: hsmmlearn's forward-backward (FBImpl.cpp), censoring 0/1. */
int tvo_fb(int censoring, int tau, int J, int M, const double* d, const double* p, const double* pi,
           const double* pdf, double* F, double* L, double* G, double* L1, double* Nn, double* Norm,
           double* eta);

#ifdef __cplusplus
}
#endif
#endif
