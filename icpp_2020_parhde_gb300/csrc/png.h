// png.h -- the library's PNG writer (png.cpp), host code only.
#pragma once
#include <cstddef>
#include <cstdint>

// Write a PNG file from ready scanlines: `rows` holds H rows of 1 + ceil(W * bits per pixel / 8) bytes, each
// starting with its filter byte.  color_type 3: palette image of the given bit depth, `palette` holds npal
// colours as 0xAABBGGRR (an alpha below 255 adds a tRNS chunk); color_type 6: 8-bit RGBA, palette unused.
// The image data is deflated by `nthreads` host threads (0: all cores).  Returns 0, or -1 when the file
// cannot be written.
int phde_png_write_rows(const char *path, const uint8_t *rows, uint32_t W, uint32_t H, int bit_depth, int color_type,
                        const uint32_t *palette, int npal, int nthreads);
