/* Declarations standing in for SEPlib's seplib.h, so that the reference's host
 * C++ compiles for the oracle's reference library (oracle/_ref).  Test infrastructure only.
 * The file-backed calls are served from an in-memory registry (sep_stubs.cpp). */
#ifndef SEPX_REF_SEPLIB_STUB_H
#define SEPX_REF_SEPLIB_STUB_H
#include <stdio.h>
#include <stdlib.h>
#ifndef MAX
#define MAX(a, b) (((a) > (b)) ? (a) : (b))
#endif
#ifndef MIN
#define MIN(a, b) (((a) < (b)) ? (a) : (b))
#endif
#ifdef __cplusplus
extern "C" {
#endif
int seperr(const char *fmt, ...);
int sreed(const char *tag, void *buf, int nbytes);
int srite(const char *tag, void *buf, int nbytes);
int sseek(const char *tag, int off, int whence);
int sseek_block(const char *tag, int block, int blocksize, int whence);
int getch(const char *name, const char *type, void *val);
int putch(const char *name, const char *type, void *val);
int auxpar(const char *name, const char *type, void *val, const char *tag);
int auxputch(const char *name, const char *type, void *val, const char *tag);
FILE *auxinout(const char *tag);
FILE *auxin(const char *tag);
FILE *auxout(const char *tag);
int auxclose(const char *tag);
int sreed_window(const char *tag, int *n_dim, int *n, int *nw, int *fw, int *jw, int esize, void *buf);
int srite_window(const char *tag, int *n_dim, int *n, int *nw, int *fw, int *jw, int esize, void *buf);
int sep_get_number_data_axes(const char *tag, int *n);
int sep_get_data_axis_par(const char *tag, int *i, int *n, float *o, float *d, char *label);
int sep_put_data_axis_par(const char *tag, int *i, int *n, float *o, float *d, char *label);
void initpar(int argc, char **argv);
#ifdef __cplusplus
}
#endif
#endif
