// stubs.cpp -- TEST INFRASTRUCTURE ONLY: libtiff and libpng calls named by
// the reference's image I/O headers (oracle/ref/shim/tiffio.h, png.h),
// defined as failures so that the reference's CPU sources link into
// oracle/_ref/ref_pin.  The driver reads and writes no TIFF or PNG file.
#include "png.h"
#include "tiffio.h"

extern "C" {
TIFF *TIFFOpen(const char *, const char *) { return nullptr; }
TIFF *TIFFClientOpen(const char *, const char *, thandle_t, TIFFReadWriteProc, TIFFReadWriteProc, TIFFSeekProc,
                     TIFFCloseProc, TIFFSizeProc, TIFFMapFileProc, TIFFUnmapFileProc) {
    return nullptr;
}
void TIFFClose(TIFF *) {}
int TIFFGetField(TIFF *, uint32_t, ...) { return 0; }
int TIFFGetFieldDefaulted(TIFF *, uint32_t, ...) { return 0; }
int TIFFSetField(TIFF *, uint32_t, ...) { return 0; }
int TIFFSetDirectory(TIFF *, uint16_t) { return 0; }
int TIFFWriteDirectory(TIFF *) { return 0; }
tsize_t TIFFStripSize(TIFF *) { return 0; }
tstrip_t TIFFNumberOfStrips(TIFF *) { return 0; }
tsize_t TIFFReadEncodedStrip(TIFF *, tstrip_t, tdata_t, tsize_t) { return -1; }
tsize_t TIFFWriteEncodedStrip(TIFF *, tstrip_t, tdata_t, tsize_t) { return -1; }
int TIFFWriteScanline(TIFF *, tdata_t, uint32_t, uint16_t) { return -1; }
tdata_t _TIFFmalloc(tsize_t) { return nullptr; }
void _TIFFfree(tdata_t) {}

int png_sig_cmp(png_bytep, size_t, size_t) { return 1; }
png_structp png_create_read_struct(const char *, void *, png_error_ptr, png_error_ptr) { return nullptr; }
png_structp png_create_write_struct(const char *, void *, png_error_ptr, png_error_ptr) { return nullptr; }
png_infop png_create_info_struct(png_structp) { return nullptr; }
void png_destroy_read_struct(png_structp *, png_infop *, png_infop *) {}
void png_destroy_write_struct(png_structp *, png_infop *) {}
void png_init_io(png_structp, FILE *) {}
void png_read_info(png_structp, png_infop) {}
png_uint_32 png_get_IHDR(png_structp, png_infop, png_uint_32 *, png_uint_32 *, int *, int *, int *, int *, int *) {
    return 0;
}
void png_set_IHDR(png_structp, png_infop, png_uint_32, png_uint_32, int, int, int, int, int) {}
void png_set_strip_16(png_structp) {}
void png_set_palette_to_rgb(png_structp) {}
void png_set_expand_gray_1_2_4_to_8(png_structp) {}
void png_set_gray_to_rgb(png_structp) {}
void png_set_filler(png_structp, png_uint_32, int) {}
int png_set_interlace_handling(png_structp) { return 0; }
void png_read_update_info(png_structp, png_infop) {}
size_t png_get_rowbytes(png_structp, png_infop) { return 0; }
void *png_malloc(png_structp, size_t) { return nullptr; }
void png_free(png_structp, void *) {}
void png_read_image(png_structp, png_bytep *) {}
void png_read_end(png_structp, png_infop) {}
void png_write_info(png_structp, png_infop) {}
void png_write_image(png_structp, png_bytep *) {}
void png_write_end(png_structp, png_infop) {}
}
