/* The part of libbench2's user interface (bench-user.h, FFTW's benchmark
 * library) that afft's libbench2 test program misc/libbench2-test/doit.cpp
 * uses, restated for the test driver tests/cxx/bench2_main.cpp: the problem
 * description the harness hands to the program's hooks, and the
 * documentation table the program defines.  libbench2 itself is not part of
 * this repository or the reference. */
#ifndef AFFT_GB300_BENCH_USER_H
#define AFFT_GB300_BENCH_USER_H

#ifdef __cplusplus
extern "C" {
#endif

/* one dimension of a tensor: length and input / output strides (elements) */
typedef struct {
  int n;
  int is;
  int os;
} bench_iodim;

typedef struct {
  int rnk;
  bench_iodim* dims;
} bench_tensor;

typedef enum { PROBLEM_COMPLEX, PROBLEM_REAL, PROBLEM_R2R } problem_kind_t;

typedef struct {
  problem_kind_t kind;
  bench_tensor* sz;     /* transform dimensions */
  bench_tensor* vecsz;  /* batch dimensions (rank 0 here) */
  int sign;             /* -1 forward, +1 backward (unnormalised) */
  int in_place;
  int destroy_input;
  int split;
  void* in;             /* interleaved complex float data */
  void* out;
  void* userinfo;
} bench_problem;

/* the program's documentation table: key/value pairs ending in a null key */
struct bench_doc {
  const char* key;
  const char* val;
  const char* (*f)(void);
};
extern struct bench_doc bench_doc[];

#ifdef __cplusplus
}
#endif

#define BEGIN_BENCH_DOC struct bench_doc bench_doc[] = {
#define BENCH_DOC(key, val) {key, val, 0},
#define BENCH_DOCF(key, f) {key, 0, f},
#define END_BENCH_DOC {0, 0, 0}};

/* the hooks a libbench2 program provides */
int can_do(bench_problem* p);
void setup(bench_problem* p);
void doit(int iter, bench_problem* p);
void done(bench_problem* p);
void cleanup(void);
void main_init(int* argc, char*** argv);

#endif
