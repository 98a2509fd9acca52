/* No-op stand-in for libpng, used only when the reference sources are
 * compiled into the test oracle (oracle/_ref).  The reference includes
 * <png.h> from PngWriter.hpp for slice images, which are outside the solver
 * path; libpng headers are not installed here.  Every call below does
 * nothing and reports failure, so PngWriter::write returns early. */
#ifndef CS3D_STUB_PNG_H
#define CS3D_STUB_PNG_H
#include <stdio.h>
typedef unsigned char png_byte;
typedef png_byte *png_bytep;
typedef png_bytep *png_bytepp;
typedef void *png_voidp;
typedef struct cs3d_png_struct *png_structp;
typedef struct cs3d_png_info *png_infop;
typedef png_structp *png_structpp;
typedef png_infop *png_infopp;
#define PNG_LIBPNG_VER_STRING "stub"
#define PNG_COLOR_TYPE_RGB 2
#define PNG_COLOR_TYPE_GRAY 0
#define PNG_INTERLACE_NONE 0
#define PNG_COMPRESSION_TYPE_DEFAULT 0
#define PNG_FILTER_TYPE_DEFAULT 0
static inline png_structp png_create_write_struct(const char *v, png_voidp e, void *f, void *w)
{ (void)v; (void)e; (void)f; (void)w; return 0; }
static inline png_infop png_create_info_struct(png_structp p) { (void)p; return 0; }
static inline void png_destroy_write_struct(png_structpp p, png_infopp i) { (void)p; (void)i; }
static inline void png_init_io(png_structp p, FILE *f) { (void)p; (void)f; }
static inline void png_set_IHDR(png_structp p, png_infop i, unsigned w, unsigned h, int b, int c,
                                int il, int cm, int fm)
{ (void)p; (void)i; (void)w; (void)h; (void)b; (void)c; (void)il; (void)cm; (void)fm; }
static inline void png_write_info(png_structp p, png_infop i) { (void)p; (void)i; }
static inline void png_write_image(png_structp p, png_bytepp r) { (void)p; (void)r; }
static inline void png_write_end(png_structp p, png_infop i) { (void)p; (void)i; }
#endif
