/* Test harness (test infrastructure only): drives a libbench2 backend's can_do / setup /
 * doit / done on one problem described by plain arrays, with the stand-in libbench2 header of
 * this folder, and provides the two libbench2 routines a backend calls. */
#include <stdlib.h>

#include "libbench2/bench-user.h"

double tensor_sz(const bench_tensor *t)
{
     double s = 1;
     int i;
     for (i = 0; i < t->rnk; ++i) s *= t->dims[i].n;
     return s;
}

static int exit_status;
void bench_exit(int status)
{
     exit_status = status ? status : 1;
}

/* kind: 0 complex, 1 real (rdft2), 2 r2r.  dims: rnk + vrnk triples (n, is, os), transform
 * dimensions first; r2r: one kind per transform dimension.  Returns 0 when the problem ran,
 * -1 when can_do refused it, the bench_exit status otherwise. */
int lfgb_run(int kind, int sign, int rnk, int vrnk, const int *dims, const int *r2r, int split,
             double *in, double *out, double *ini, double *outi, int iphyssz, int ophyssz,
             int iter)
{
     bench_iodim d[16];
     bench_tensor sz, vecsz;
     r2r_kind_t k[8];
     bench_problem p;
     int i;
     if (rnk + vrnk > 16 || rnk > 8) return -2;
     for (i = 0; i < rnk + vrnk; ++i) {
          d[i].n = dims[3 * i];
          d[i].is = dims[3 * i + 1];
          d[i].os = dims[3 * i + 2];
     }
     for (i = 0; i < rnk; ++i) k[i] = r2r ? (r2r_kind_t) r2r[i] : R2R_R2HC;
     sz.rnk = rnk;
     sz.dims = d;
     vecsz.rnk = vrnk;
     vecsz.dims = d + rnk;
     p.kind = kind == 0 ? PROBLEM_COMPLEX : kind == 1 ? PROBLEM_REAL : PROBLEM_R2R;
     p.k = k;
     p.sz = &sz;
     p.vecsz = &vecsz;
     p.sign = sign;
     p.in_place = in == out;
     p.destroy_input = 0;
     p.split = split;
     p.in = in;
     p.out = out;
     p.inphys = in;
     p.outphys = out;
     p.iphyssz = iphyssz;
     p.ophyssz = ophyssz;
     p.pstring = 0;
     p.userinfo = 0;
     p.scrambled_in = p.scrambled_out = 0;
     p.ini = ini;
     p.outi = outi;
     exit_status = 0;
     if (!can_do(&p)) return -1;
     setup(&p);
     if (exit_status) return exit_status;
     doit(iter, &p);
     done(&p);
     return exit_status;
}
