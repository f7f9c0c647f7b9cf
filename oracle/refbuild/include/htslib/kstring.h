/* Clean-room subset of htslib's kstring API (see hts.h).  Test infrastructure. */
#ifndef BSQ_REF_KSTRING_H
#define BSQ_REF_KSTRING_H

#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct kstring_t {
  size_t l, m;
  char* s;
} kstring_t;

#define KS_INITIALIZE {0, 0, NULL}

static inline int ks_resize(kstring_t* s, size_t size) {
  if (s->m < size) {
    size_t m = size + (size >> 1) + 16;
    char* p = (char*)realloc(s->s, m);
    if (!p) return -1;
    s->s = p;
    s->m = m;
  }
  return 0;
}

static inline int kputsn(const char* p, size_t l, kstring_t* s) {
  if (ks_resize(s, s->l + l + 1) < 0) return EOF;
  memcpy(s->s + s->l, p, l);
  s->l += l;
  s->s[s->l] = 0;
  return (int)l;
}

static inline int kputs(const char* p, kstring_t* s) { return kputsn(p, strlen(p), s); }

static inline void ks_free(kstring_t* s) {
  if (s) {
    free(s->s);
    s->s = NULL;
    s->l = s->m = 0;
  }
}

#ifdef __cplusplus
}
#endif
#endif
