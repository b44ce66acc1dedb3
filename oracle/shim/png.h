/* libpng declarations stand-in (TEST INFRASTRUCTURE): the reference's PNG
 * writer is dead code that is not compiled here, but one of its headers is
 * included on the way to the DFT class, so its types must exist. */
#ifndef DFTG_SHIM_PNG_H
#define DFTG_SHIM_PNG_H
#include <stddef.h>
typedef struct png_struct_def png_struct;
typedef png_struct *png_structp;
typedef unsigned char png_byte;
typedef png_byte *png_bytep;
typedef size_t png_size_t;
#endif
