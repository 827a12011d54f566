/* sepx_sepio.h -- SEP regular datasets (header "name.H" + binary data file)
 * read into and written from host or device float buffers.
 *
 * The reference reads and writes these through SEPlib (Born/sreg.cpp:17-102
 * tag_init / read_axis / get_int / get_float / get_string, Born/sregf.cpp
 * read_all / write_all / read_slice / write_slice); this library implements
 * the format itself: key=value headers (a later value of a key overrides an
 * earlier one), n1..n8 / o / d / label axes, esize=4, data_format "xdr_float"
 * (big-endian, the default) or "native_float", in= data file.
 *
 * Every function returns 0 or a non-zero status with the message in
 * sepx_last_error().  on_device != 0: the buffer is a device pointer and the
 * transfer runs on the library's stream (setup_cuda first; the call returns
 * when the data is in place).  Not re-entrant: calls share one pair of pinned
 * staging buffers. */
#ifndef SEPX_SEPIO_H
#define SEPX_SEPIO_H

#ifdef __cplusplus
extern "C" {
#endif

#define SEPX_SEP_MAX_AXES 8

/* sreg::tag_init + read_axis: number of axes (largest i with n_i > 1) and
 * n / o / d of all eight (unset: 1 / 0 / 1); any pointer may be NULL */
int sepx_sep_info(const char *header, int *ndim, int n[8], float o[8], float d[8]);
/* sreg::get_string: the value of `key` (0), 1 if the header does not set it */
int sepx_sep_par(const char *header, const char *key, char *out, int cap);
/* sregf::read_all / read_next: `count` elements from element `first` of the
 * data (axis 1 fastest) */
int sepx_sep_read(const char *header, long long first, long long count, float *dst, int on_device);
/* sregf::read_slice: the window nw (sizes), fw (first index, NULL: 0), jw
 * (step, NULL: 1) of all eight axes, written densely */
int sepx_sep_read_window(const char *header, const int *nw, const int *fw, const int *jw, float *dst,
                         int on_device);
/* sreg::write_description + sregf::write_all: header `header` and data file
 * `header`@ (overwritten); labels: newline-separated axis labels or NULL;
 * xdr != 0 writes big-endian xdr_float, 0 native_float */
int sepx_sep_write(const char *header, int ndim, const int *n, const float *o, const float *d,
                   const char *labels, const float *src, int on_device, int xdr);

#ifdef __cplusplus
}
#endif
#endif
