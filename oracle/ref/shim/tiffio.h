/*
 * tiffio.h -- TEST INFRASTRUCTURE ONLY: type and function declarations of the
 * libtiff interface that the reference's src/image.h and src/rwTIFF.h name,
 * so that the reference's CPU sources compile into the oracle's reference
 * build.  libtiff is not installed here and the oracle reads no TIFF file:
 * oracle/ref/stubs.cpp implements every function as a failure (NULL / 0).
 */
#ifndef GBR_ORACLE_TIFFIO_SHIM_H
#define GBR_ORACLE_TIFFIO_SHIM_H
#include <stddef.h>
#include <stdint.h>
#include <sys/types.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct gbr_shim_tiff TIFF;
typedef int64_t tsize_t;
typedef uint64_t toff_t;
typedef void *tdata_t;
typedef void *thandle_t;
typedef uint32_t tstrip_t;
typedef uint16_t uint16;
typedef uint32_t uint32;
typedef tsize_t (*TIFFReadWriteProc)(thandle_t, tdata_t, tsize_t);
typedef toff_t (*TIFFSeekProc)(thandle_t, toff_t, int);
typedef int (*TIFFCloseProc)(thandle_t);
typedef toff_t (*TIFFSizeProc)(thandle_t);
typedef int (*TIFFMapFileProc)(thandle_t, tdata_t *, toff_t *);
typedef void (*TIFFUnmapFileProc)(thandle_t, tdata_t, toff_t);

#define TIFFTAG_IMAGEWIDTH 256
#define TIFFTAG_IMAGELENGTH 257
#define TIFFTAG_BITSPERSAMPLE 258
#define TIFFTAG_COMPRESSION 259
#define TIFFTAG_PHOTOMETRIC 262
#define TIFFTAG_ORIENTATION 274
#define TIFFTAG_SAMPLESPERPIXEL 277
#define TIFFTAG_ROWSPERSTRIP 278
#define TIFFTAG_XRESOLUTION 282
#define TIFFTAG_YRESOLUTION 283
#define TIFFTAG_PLANARCONFIG 284
#define TIFFTAG_RESOLUTIONUNIT 296
#define TIFFTAG_SOFTWARE 305
#define TIFFTAG_SAMPLEFORMAT 339
#define SAMPLEFORMAT_UINT 1
#define SAMPLEFORMAT_INT 2
#define SAMPLEFORMAT_IEEEFP 3
#define RESUNIT_NONE 1
#define RESUNIT_INCH 2
#define RESUNIT_CENTIMETER 3
#define ORIENTATION_TOPLEFT 1
#define PHOTOMETRIC_MINISBLACK 1
#define PLANARCONFIG_CONTIG 1
#define COMPRESSION_NONE 1
#define COMPRESSION_LZW 5
#define COMPRESSION_DEFLATE 32946

TIFF *TIFFOpen(const char *name, const char *mode);
TIFF *TIFFClientOpen(const char *name, const char *mode, thandle_t h, TIFFReadWriteProc rd,
                     TIFFReadWriteProc wr, TIFFSeekProc sk, TIFFCloseProc cl, TIFFSizeProc sz,
                     TIFFMapFileProc mp, TIFFUnmapFileProc ump);
void TIFFClose(TIFF *t);
int TIFFGetField(TIFF *t, uint32_t tag, ...);
int TIFFGetFieldDefaulted(TIFF *t, uint32_t tag, ...);
int TIFFSetField(TIFF *t, uint32_t tag, ...);
int TIFFSetDirectory(TIFF *t, uint16_t dir);
int TIFFWriteDirectory(TIFF *t);
tsize_t TIFFStripSize(TIFF *t);
tstrip_t TIFFNumberOfStrips(TIFF *t);
tsize_t TIFFReadEncodedStrip(TIFF *t, tstrip_t s, tdata_t buf, tsize_t size);
tsize_t TIFFWriteEncodedStrip(TIFF *t, tstrip_t s, tdata_t buf, tsize_t size);
int TIFFWriteScanline(TIFF *t, tdata_t buf, uint32_t row, uint16_t sample);
tdata_t _TIFFmalloc(tsize_t n);
void _TIFFfree(tdata_t p);
#ifdef __cplusplus
}
#endif
#endif
