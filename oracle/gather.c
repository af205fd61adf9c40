/*
 * oracle/gather.c -- CPU restatement of LibreTT's transpose semantics.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline legs may load this library, and only as the checker
 * or as the timed host loop; the engine never calls it.
 *
 * Semantics (LibreTT tests/example.cpp:170-212): tensors are column-major; with
 * abc[i] = prod_{j<i} dim[j] and cba[i] = prod_{j<i} dim[perm[j]],
 *     out[sum_r cba[r] * idx[perm[r]]] = in[sum_r abc[r] * idx[r]].
 * Elements are copied as raw 4/8/16-byte words.
 *
 * oracle_check_pattern restates LibreTT's device checker
 * (src/TensorTester.cpp:47-126 with the constants of calcTensorConv,
 * src/TensorTester.cpp:201-220): when the input holds the 32-bit word pattern
 * word[w] = w (src/TensorTester.cpp:34-40), the low 32 bits of output element
 * i divided by sizeofType/4 must equal sum_r ((i / c_r) % d_r) * ct_r with
 * c_r = output stride of input rank r, d_r = dim[r], ct_r = input stride.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_MAXR 32

typedef struct {
  const unsigned char* in;
  unsigned char* out;
  int rank;
  int esize;
  int64_t odim[ORACLE_MAXR];  /* output-order dims */
  int64_t istr[ORACLE_MAXR];  /* input stride of output-order rank k (elements) */
  int64_t begin, end;         /* output element range */
} slab_t;

static void* run_slab(void* arg) {
  slab_t* s = (slab_t*)arg;
  int64_t idx[ORACLE_MAXR];
  int64_t rem = s->begin, src = 0;
  for (int k = 0; k < s->rank; ++k) {
    idx[k] = rem % s->odim[k];
    rem /= s->odim[k];
    src += idx[k] * s->istr[k];
  }
  const int es = s->esize;
  for (int64_t o = s->begin; o < s->end; ++o) {
    const unsigned char* from = s->in + src * es;
    unsigned char* to = s->out + o * es;
    if (es == 4) {
      uint32_t v;
      memcpy(&v, from, 4);
      memcpy(to, &v, 4);
    } else if (es == 8) {
      uint64_t v;
      memcpy(&v, from, 8);
      memcpy(to, &v, 8);
    } else {
      uint64_t v[2];
      memcpy(v, from, 16);
      memcpy(to, v, 16);
    }
    /* odometer over output coordinates */
    for (int k = 0; k < s->rank; ++k) {
      src += s->istr[k];
      if (++idx[k] < s->odim[k]) break;
      src -= idx[k] * s->istr[k];
      idx[k] = 0;
    }
  }
  return NULL;
}

/* Returns 0 on success, -1 on invalid arguments. */
int oracle_transpose(const void* in, void* out, int rank, const int* dim, const int* perm,
                     int esize, int nthreads) {
  if (rank < 1 || rank > ORACLE_MAXR || (esize != 4 && esize != 8 && esize != 16)) return -1;
  int64_t abc[ORACLE_MAXR];
  int64_t vol = 1;
  for (int r = 0; r < rank; ++r) {
    if (dim[r] < 1) return -1;
    abc[r] = vol;
    vol *= dim[r];
  }
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  if ((int64_t)nthreads > vol) nthreads = (int)vol;
  slab_t* slabs = (slab_t*)calloc((size_t)nthreads, sizeof(slab_t));
  pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
  if (!slabs || !th) {
    free(slabs);
    free(th);
    return -1;
  }
  for (int t = 0; t < nthreads; ++t) {
    slab_t* s = &slabs[t];
    s->in = (const unsigned char*)in;
    s->out = (unsigned char*)out;
    s->rank = rank;
    s->esize = esize;
    for (int k = 0; k < rank; ++k) {
      if (perm[k] < 0 || perm[k] >= rank) {
        free(slabs);
        free(th);
        return -1;
      }
      s->odim[k] = dim[perm[k]];
      s->istr[k] = abc[perm[k]];
    }
    s->begin = vol * t / nthreads;
    s->end = vol * (t + 1) / nthreads;
  }
  int started = 0;
  for (int t = 1; t < nthreads; ++t) {
    if (pthread_create(&th[t], NULL, run_slab, &slabs[t]) != 0) break;
    started = t;
  }
  run_slab(&slabs[0]);
  for (int t = 1; t <= started; ++t) pthread_join(th[t], NULL);
  for (int t = started + 1; t < nthreads; ++t) run_slab(&slabs[t]);
  free(slabs);
  free(th);
  return 0;
}

/* word[w] = w for w in [0, nwords) (LibreTT src/TensorTester.cpp:34-40). */
void oracle_fill_pattern(uint32_t* words, int64_t nwords) {
  for (int64_t w = 0; w < nwords; ++w) words[w] = (uint32_t)w;
}

/*
 * Returns the first output position whose pattern does not match, or -1 if
 * all match; -2 on invalid arguments.  *ref_val / *data_val receive the
 * expected and found values at that position.
 */
int64_t oracle_check_pattern(const void* out, int rank, const int* dim, const int* perm,
                             int esize, int64_t* ref_val, int64_t* data_val) {
  if (rank < 1 || rank > ORACLE_MAXR || (esize != 4 && esize != 8 && esize != 16)) return -2;
  int64_t c[ORACLE_MAXR], d[ORACLE_MAXR], ct[ORACLE_MAXR];
  int64_t vol = 1;
  for (int r = 0; r < rank; ++r) {
    d[r] = dim[r];
    ct[r] = vol;
    vol *= dim[r];
  }
  c[perm[0]] = 1;
  for (int i = 1; i < rank; ++i) c[perm[i]] = c[perm[i - 1]] * dim[perm[i - 1]];
  const unsigned char* o = (const unsigned char*)out;
  const int64_t per = esize / 4;
  for (int64_t i = 0; i < vol; ++i) {
    int64_t ref = 0;
    for (int r = 0; r < rank; ++r) ref += ((i / c[r]) % d[r]) * ct[r];
    uint32_t low;
    memcpy(&low, o + i * esize, 4);
    int64_t val = (int64_t)low / per;
    if (val != ref) { /* pattern words are unique while vol * esize / 4 < 2^32 */
      if (ref_val) *ref_val = ref;
      if (data_val) *data_val = val;
      return i;
    }
  }
  return -1;
}
