/*
 * png.h -- TEST INFRASTRUCTURE ONLY: declarations of the libpng calls that
 * the reference's src/jaz/gravis/private/tImageIO_PNG.hxx names, so that the
 * reference's CPU sources compile into the oracle's reference build.
 * libpng is not installed here and the oracle writes no PNG file:
 * oracle/ref/stubs.cpp implements the calls as failures.
 */
#ifndef GBR_ORACLE_PNG_SHIM_H
#define GBR_ORACLE_PNG_SHIM_H
#include <stddef.h>
#include <stdio.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef unsigned char png_byte;
typedef png_byte *png_bytep;
typedef unsigned int png_uint_32;
typedef struct gbr_shim_png_struct png_struct;
typedef png_struct *png_structp;
typedef struct gbr_shim_png_info png_info;
typedef png_info *png_infop;
typedef void (*png_error_ptr)(png_structp, const char *);

#define PNG_LIBPNG_VER_STRING "0.0.0-shim"
#define PNG_COLOR_TYPE_GRAY 0
#define PNG_COLOR_TYPE_PALETTE 3
#define PNG_COLOR_TYPE_RGB 2
#define PNG_COLOR_TYPE_RGB_ALPHA 6
#define PNG_COMPRESSION_TYPE_BASE 0
#define PNG_FILTER_TYPE_BASE 0
#define PNG_INTERLACE_NONE 0
#define PNG_FILLER_AFTER 1

int png_sig_cmp(png_bytep sig, size_t start, size_t n);
png_structp png_create_read_struct(const char *ver, void *err_ptr, png_error_ptr err_fn, png_error_ptr warn_fn);
png_structp png_create_write_struct(const char *ver, void *err_ptr, png_error_ptr err_fn, png_error_ptr warn_fn);
png_infop png_create_info_struct(png_structp p);
void png_destroy_read_struct(png_structp *p, png_infop *i, png_infop *e);
void png_destroy_write_struct(png_structp *p, png_infop *i);
void png_init_io(png_structp p, FILE *f);
void png_read_info(png_structp p, png_infop i);
png_uint_32 png_get_IHDR(png_structp p, png_infop i, png_uint_32 *w, png_uint_32 *h, int *depth, int *color,
                         int *interlace, int *compression, int *filter);
void png_set_IHDR(png_structp p, png_infop i, png_uint_32 w, png_uint_32 h, int depth, int color, int interlace,
                  int compression, int filter);
void png_set_strip_16(png_structp p);
void png_set_palette_to_rgb(png_structp p);
void png_set_expand_gray_1_2_4_to_8(png_structp p);
void png_set_gray_to_rgb(png_structp p);
void png_set_filler(png_structp p, png_uint_32 filler, int flags);
int png_set_interlace_handling(png_structp p);
void png_read_update_info(png_structp p, png_infop i);
size_t png_get_rowbytes(png_structp p, png_infop i);
void *png_malloc(png_structp p, size_t n);
void png_free(png_structp p, void *ptr);
void png_read_image(png_structp p, png_bytep *rows);
void png_read_end(png_structp p, png_infop i);
void png_write_info(png_structp p, png_infop i);
void png_write_image(png_structp p, png_bytep *rows);
void png_write_end(png_structp p, png_infop i);
#ifdef __cplusplus
}
#endif
#endif
