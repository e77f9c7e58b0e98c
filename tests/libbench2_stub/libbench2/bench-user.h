/* Test stand-in for libbench2's bench-user.h (FFTW 3.3.10, not vendored here): only the
 * declarations a libbench2 backend uses, with libbench2's names, so that
 * lean-fftw_gb300/csrc/tools/bench_lfg.c compiles and can be driven without libbench2
 * (tests/libbench2_stub/harness.c).  Built against the real header, the backend links into
 * libbench2's benchmark program unchanged. */
#ifndef LFG_TEST_BENCH_USER_H
#define LFG_TEST_BENCH_USER_H

#include <limits.h>
#include <stddef.h>

typedef double bench_real;
typedef bench_real bench_complex[2];

typedef struct {
     int n;          /* dimension size */
     int is;         /* input stride, in bench_real (complex data: in complex elements) */
     int os;         /* output stride */
} bench_iodim;

typedef struct {
     int rnk;
     bench_iodim *dims;
} bench_tensor;

#define RNK_MINFTY INT_MAX
#define BENCH_FINITE_RNK(rnk) ((rnk) != RNK_MINFTY)

typedef enum { PROBLEM_COMPLEX, PROBLEM_REAL, PROBLEM_R2R } problem_kind_t;

typedef enum {
     R2R_R2HC, R2R_HC2R, R2R_DHT,
     R2R_REDFT00, R2R_REDFT01, R2R_REDFT10, R2R_REDFT11,
     R2R_RODFT00, R2R_RODFT01, R2R_RODFT10, R2R_RODFT11
} r2r_kind_t;

typedef struct {
     problem_kind_t kind;
     r2r_kind_t *k;
     bench_tensor *sz;
     bench_tensor *vecsz;
     int sign;
     int in_place;
     int destroy_input;
     int split;
     void *in, *out;
     void *inphys, *outphys;
     int iphyssz, ophyssz;
     char *pstring;
     void *userinfo;
     int scrambled_in, scrambled_out;
     void *ini, *outi;    /* split format: imaginary bases (NULL: re base + phys size) */
} bench_problem;

struct bench_doc {
     const char *key;
     const char *val;
     const char *(*f)(void);
};
#define BEGIN_BENCH_DOC const struct bench_doc bench_doc[] = {
#define BENCH_DOC(key, val) { key, val, 0 },
#define END_BENCH_DOC { 0, 0, 0 } };

/* provided by libbench2 (here by the test harness) */
extern double tensor_sz(const bench_tensor *t);
extern void bench_exit(int status);

/* provided by the backend */
extern int can_do(bench_problem *p);
extern void setup(bench_problem *p);
extern void doit(int iter, bench_problem *p);
extern void done(bench_problem *p);
extern void main_init(int *argc, char ***argv);
extern void initial_cleanup(void);
extern void final_cleanup(void);

#endif
