// png.cpp -- PNG output for the drawing tool: the reference writes its image with lodepng_encode32_file
// (draw_graph.c:331); this writer produces a PNG of the same pixels, deflated by many host threads.
//
// Format: PNG (ISO/IEC 15948) with a zlib stream (RFC 1950) of deflate data (RFC 1951).  The scanlines are
// cut into ranges that threads compress independently with fixed-Huffman blocks; a match may still reach back
// into the previous range (the decoder keeps a 32 KiB window across blocks), so cutting costs almost nothing.
// Each range ends with an empty stored block, which byte-aligns it, and becomes its own IDAT chunk with its
// own CRC; the Adler-32 of the whole stream is combined from the ranges' partial sums.  Matches are found
// among three candidates per position: the previous byte (runs), the byte one scanline up, and the last
// position with the same 4-byte hash.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "parhde.h"
#include "png.h"

namespace {

constexpr uint32_t ADLER_MOD = 65521;
constexpr int WINDOW = 32768;
constexpr int MAX_MATCH = 258;
constexpr int HASH_BITS = 16;

struct CrcTable {
  uint32_t t[256];
  CrcTable() {
    for (uint32_t n = 0; n < 256; n++) {
      uint32_t c = n;
      for (int k = 0; k < 8; k++) c = (c & 1) ? 0xedb88320u ^ (c >> 1) : c >> 1;
      t[n] = c;
    }
  }
};
const CrcTable &crc_table() {
  static const CrcTable tab;
  return tab;
}
uint32_t crc_update(uint32_t crc, const uint8_t *p, size_t n) {
  const uint32_t *t = crc_table().t;
  uint32_t c = crc ^ 0xffffffffu;
  for (size_t i = 0; i < n; i++) c = t[(c ^ p[i]) & 0xff] ^ (c >> 8);
  return c ^ 0xffffffffu;
}

// Adler-32 pieces of a range: a = sum of bytes, b = sum of running sums (both from 0), mod 65521.
struct AdlerPart {
  uint32_t a = 0, b = 0;
  size_t n = 0;
};
AdlerPart adler_part(const uint8_t *p, size_t n) {
  AdlerPart r;
  r.n = n;
  uint64_t a = 0, b = 0;
  for (size_t i = 0; i < n;) {
    const size_t stop = std::min(n, i + (size_t(1) << 16));  // b stays far below 2^64 within a block
    for (; i < stop; i++) {
      a += p[i];
      b += a;
    }
    a %= ADLER_MOD;
    b %= ADLER_MOD;
  }
  r.a = (uint32_t)a;
  r.b = (uint32_t)b;
  return r;
}

// Fixed-Huffman codes (RFC 1951 3.2.6), bit-reversed for the LSB-first bit stream.
struct FixedCodes {
  uint16_t lit_code[288];
  uint8_t lit_len[288];
  uint16_t len_sym[MAX_MATCH + 1];  // match length -> symbol 257..285
  uint8_t len_extra_bits[MAX_MATCH + 1];
  uint16_t len_extra_val[MAX_MATCH + 1];
  uint8_t dist_code_rev[30];
  static uint32_t rev(uint32_t v, int n) {
    uint32_t r = 0;
    for (int i = 0; i < n; i++) r |= ((v >> i) & 1u) << (n - 1 - i);
    return r;
  }
  FixedCodes() {
    for (int s = 0; s < 288; s++) {
      uint32_t code;
      int len;
      if (s < 144) code = 0x30 + s, len = 8;
      else if (s < 256) code = 0x190 + (s - 144), len = 9;
      else if (s < 280) code = s - 256, len = 7;
      else code = 0xc0 + (s - 280), len = 8;
      lit_code[s] = (uint16_t)rev(code, len);
      lit_len[s] = (uint8_t)len;
    }
    int base = 3;
    for (int c = 257; c <= 284; c++) {
      const int extra = c < 265 ? 0 : (c - 261) / 4;
      for (int l = base; l < base + (1 << extra) && l < MAX_MATCH; l++) {
        len_sym[l] = (uint16_t)c;
        len_extra_bits[l] = (uint8_t)extra;
        len_extra_val[l] = (uint16_t)(l - base);
      }
      base += 1 << extra;
    }
    len_sym[MAX_MATCH] = 285;  // 258 has its own symbol
    len_extra_bits[MAX_MATCH] = 0;
    len_extra_val[MAX_MATCH] = 0;
    for (int c = 0; c < 30; c++) dist_code_rev[c] = (uint8_t)rev((uint32_t)c, 5);
  }
};
const FixedCodes &codes() {
  static const FixedCodes tab;
  return tab;
}

struct BitOut {
  std::vector<uint8_t> &buf;
  uint64_t acc = 0;
  int nb = 0;
  explicit BitOut(std::vector<uint8_t> &b) : buf(b) {}
  void put(uint32_t v, int n) {  // n <= 32
    acc |= (uint64_t)v << nb;
    nb += n;
    if (nb >= 32) {
      for (int i = 0; i < 4; i++) buf.push_back((uint8_t)(acc >> (8 * i)));
      acc >>= 32;
      nb -= 32;
    }
  }
  void align() {  // pad with zero bits to a byte boundary and flush
    while (nb > 0) {
      buf.push_back((uint8_t)acc);
      acc >>= 8;
      nb -= 8;
    }
    nb = 0;
    acc = 0;
  }
};

inline uint32_t load32(const uint8_t *p) {
  uint32_t v;
  memcpy(&v, p, 4);
  return v;
}

// Length of the common prefix of a and b, at most maxlen.
inline int match_length(const uint8_t *a, const uint8_t *b, int maxlen) {
  int l = 0;
  while (l + 8 <= maxlen) {
    uint64_t x, y;
    memcpy(&x, a + l, 8);
    memcpy(&y, b + l, 8);
    if (x != y) {
      int byte = 0;  // first differing byte in memory order, independent of the host byte order
      while (a[l + byte] == b[l + byte]) byte++;
      return l + byte;
    }
    l += 8;
  }
  while (l < maxlen && a[l] == b[l]) l++;
  return l;
}

// Deflate data[beg, end) (matches may reach back to data[0]) as one fixed-Huffman block followed by an empty
// stored block; appends whole bytes to out.
void deflate_range(const uint8_t *data, size_t size, size_t beg, size_t end, size_t stride, std::vector<uint8_t> &out) {
  const FixedCodes &fc = codes();
  BitOut bo(out);
  bo.put(2, 3);  // BFINAL 0, BTYPE 01
  std::vector<int64_t> head(size_t(1) << HASH_BITS, -1);
  auto hash_at = [&](size_t i) -> uint32_t { return (load32(data + i) * 2654435761u) >> (32 - HASH_BITS); };
  // positions up to WINDOW before beg seed the hash table, so the first matches can reach back
  for (size_t i = beg > (size_t)WINDOW ? beg - WINDOW : 0; i < beg && i + 4 <= size; i++) head[hash_at(i)] = (int64_t)i;
  size_t i = beg;
  while (i < end) {
    const int maxlen = (int)std::min<size_t>(MAX_MATCH, end - i);
    int best = 0;
    size_t bestd = 0;
    if (maxlen >= 3) {
      auto consider = [&](size_t d) {
        if (d == 0 || d > (size_t)WINDOW || d > i) return;
        const int l = match_length(data + i - d, data + i, maxlen);
        if (l > best || (l == best && d < bestd)) {
          best = l;
          bestd = d;
        }
      };
      consider(1);
      if (stride > 1) consider(stride);
      if (i + 4 <= size) {
        const uint32_t h = hash_at(i);
        const int64_t c = head[h];
        if (c >= 0) consider(i - (size_t)c);
        head[h] = (int64_t)i;
      }
    } else if (i + 4 <= size) {
      head[hash_at(i)] = (int64_t)i;
    }
    if (best >= 3) {
      const int sym = fc.len_sym[best];
      bo.put(fc.lit_code[sym], fc.lit_len[sym]);
      if (fc.len_extra_bits[best]) bo.put(fc.len_extra_val[best], fc.len_extra_bits[best]);
      const uint32_t x = (uint32_t)(bestd - 1);
      int dc, eb;
      uint32_t ev;
      if (x < 4) {
        dc = (int)x;
        eb = 0;
        ev = 0;
      } else {
        int nb = 31 - __builtin_clz(x);  // floor(log2 x) >= 2
        const uint32_t bit = (x >> (nb - 1)) & 1u;
        dc = 2 * nb + (int)bit;
        eb = nb - 1;
        ev = x - ((2u | bit) << (nb - 1));
      }
      bo.put(fc.dist_code_rev[dc], 5);
      if (eb) bo.put(ev, eb);
      // index a few positions inside the match for later hash candidates
      const size_t stop = std::min<size_t>(i + std::min(best, 32), size >= 4 ? size - 3 : 0);
      for (size_t j = i + 1; j < stop; j++) head[hash_at(j)] = (int64_t)j;
      i += (size_t)best;
    } else {
      bo.put(fc.lit_code[data[i]], fc.lit_len[data[i]]);
      i++;
    }
  }
  bo.put(fc.lit_code[256], fc.lit_len[256]);  // end of block
  bo.put(0, 3);                               // BFINAL 0, BTYPE 00: empty stored block
  bo.align();
  const uint8_t stored[4] = {0x00, 0x00, 0xff, 0xff};
  out.insert(out.end(), stored, stored + 4);
}

void put_be32(std::vector<uint8_t> &v, uint32_t x) {
  v.push_back((uint8_t)(x >> 24));
  v.push_back((uint8_t)(x >> 16));
  v.push_back((uint8_t)(x >> 8));
  v.push_back((uint8_t)x);
}

bool write_chunk(FILE *f, const char type[4], const uint8_t *data, size_t n, uint32_t crc_of_data_or_0, bool have_crc) {
  uint8_t hdr[8] = {(uint8_t)(n >> 24), (uint8_t)(n >> 16), (uint8_t)(n >> 8), (uint8_t)n,
                    (uint8_t)type[0], (uint8_t)type[1], (uint8_t)type[2], (uint8_t)type[3]};
  uint32_t crc = have_crc ? crc_of_data_or_0 : crc_update(crc_update(0, hdr + 4, 4), data, n);
  const uint8_t tail[4] = {(uint8_t)(crc >> 24), (uint8_t)(crc >> 16), (uint8_t)(crc >> 8), (uint8_t)crc};
  return fwrite(hdr, 1, 8, f) == 8 && (n == 0 || fwrite(data, 1, n, f) == n) && fwrite(tail, 1, 4, f) == 4;
}

}  // namespace

int phde_png_write_rows(const char *path, const uint8_t *rows, uint32_t W, uint32_t H, int bit_depth, int color_type,
                        const uint32_t *palette, int npal, int nthreads) {
  if (!path || !rows || W == 0 || H == 0) return -1;
  const int chans = color_type == 6 ? 4 : 1;
  const size_t stride = 1 + ((size_t)W * (size_t)(bit_depth * chans) + 7) / 8;
  const size_t total = stride * H;
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  const size_t min_range = size_t(1) << 18;
  const size_t nr = std::max<size_t>(1, std::min<size_t>((total + min_range - 1) / min_range, (size_t)nthreads * 4));
  const size_t per = (total + nr - 1) / nr;
  std::vector<std::vector<uint8_t>> comp(nr);
  std::vector<uint32_t> crcs(nr);
  std::vector<AdlerPart> parts(nr);
  std::atomic<size_t> next(0);
  auto work = [&]() {
    for (size_t r; (r = next.fetch_add(1)) < nr;) {
      const size_t beg = r * per, end = std::min(total, beg + per);
      comp[r].reserve((end - beg) / 8 + 64);
      deflate_range(rows, total, beg, end, stride, comp[r]);
      crcs[r] = crc_update(crc_update(0, (const uint8_t *)"IDAT", 4), comp[r].data(), comp[r].size());
      parts[r] = adler_part(rows + beg, end - beg);
    }
  };
  {
    std::vector<std::thread> pool;
    const int nt = (int)std::min<size_t>((size_t)nthreads, nr);
    for (int t = 1; t < nt; t++) pool.emplace_back(work);
    work();
    for (auto &th : pool) th.join();
  }
  uint32_t s1 = 1, s2 = 0;
  for (const AdlerPart &p : parts) {
    s2 = (uint32_t)((s2 + (uint64_t)(p.n % ADLER_MOD) * s1 + p.b) % ADLER_MOD);
    s1 = (s1 + p.a) % ADLER_MOD;
  }
  const uint32_t adler = (s2 << 16) | s1;

  FILE *f = fopen(path, "wb");
  if (!f) return -1;
  bool ok = true;
  static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
  ok = ok && fwrite(sig, 1, 8, f) == 8;
  std::vector<uint8_t> ihdr;
  put_be32(ihdr, W);
  put_be32(ihdr, H);
  ihdr.push_back((uint8_t)bit_depth);
  ihdr.push_back((uint8_t)color_type);
  ihdr.push_back(0);  // deflate
  ihdr.push_back(0);  // adaptive filtering (each row's filter byte)
  ihdr.push_back(0);  // not interlaced
  ok = ok && write_chunk(f, "IHDR", ihdr.data(), ihdr.size(), 0, false);
  if (color_type == 3) {
    std::vector<uint8_t> plte, trns;
    bool any_alpha = false;
    for (int i = 0; i < npal; i++) {
      plte.push_back((uint8_t)palette[i]);
      plte.push_back((uint8_t)(palette[i] >> 8));
      plte.push_back((uint8_t)(palette[i] >> 16));
      trns.push_back((uint8_t)(palette[i] >> 24));
      any_alpha = any_alpha || (palette[i] >> 24) != 255u;
    }
    ok = ok && write_chunk(f, "PLTE", plte.data(), plte.size(), 0, false);
    if (any_alpha) ok = ok && write_chunk(f, "tRNS", trns.data(), trns.size(), 0, false);
  }
  static const uint8_t zhdr[2] = {0x78, 0x01};  // deflate, 32 KiB window, no dictionary
  ok = ok && write_chunk(f, "IDAT", zhdr, 2, 0, false);
  for (size_t r = 0; r < nr && ok; r++) ok = write_chunk(f, "IDAT", comp[r].data(), comp[r].size(), crcs[r], true);
  std::vector<uint8_t> ztail = {0x03, 0x00};  // final empty fixed-Huffman block
  put_be32(ztail, adler);
  ok = ok && write_chunk(f, "IDAT", ztail.data(), ztail.size(), 0, false);
  ok = ok && write_chunk(f, "IEND", nullptr, 0, 0, false);
  ok = (fclose(f) == 0) && ok;
  return ok ? 0 : -1;
}

// ------------------------------------------------------------------------------------------------
// A PNG of any RGBA image: a palette image when it has at most 256 colours (1, 2, 4 or 8 bits per pixel,
// palette in increasing colour order), else 8-bit RGBA.  Rows are converted by the threads in parallel.
extern "C" int phde_write_png(const char *path, const uint8_t *rgba, uint32_t width, uint32_t height, int nthreads) {
  if (!path || !rgba || width == 0 || height == 0) return PHDE_ERR_INVALID;
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  const size_t W = width, H = height;
  const int nt = (int)std::max<size_t>(1, std::min<size_t>((size_t)nthreads, H));
  // distinct colours (up to 257) per thread, then merged
  std::vector<std::vector<uint32_t>> seen(nt);
  auto rows_of = [&](int t, size_t &y0, size_t &y1) {
    y0 = H * (size_t)t / (size_t)nt;
    y1 = H * (size_t)(t + 1) / (size_t)nt;
  };
  auto collect = [&](int t) {
    size_t y0, y1;
    rows_of(t, y0, y1);
    std::vector<uint32_t> &s = seen[t];
    uint32_t last = 0;
    bool have = false;
    for (size_t p = y0 * W; p < y1 * W && s.size() <= 256; p++) {
      uint32_t c;
      memcpy(&c, rgba + 4 * p, 4);
      if (have && c == last) continue;
      if (std::find(s.begin(), s.end(), c) == s.end()) s.push_back(c);
      last = c;
      have = true;
    }
  };
  {
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; t++) pool.emplace_back(collect, t);
    collect(0);
    for (auto &th : pool) th.join();
  }
  std::vector<uint32_t> pal;
  for (auto &s : seen) pal.insert(pal.end(), s.begin(), s.end());
  std::sort(pal.begin(), pal.end());
  pal.erase(std::unique(pal.begin(), pal.end()), pal.end());
  const bool palette = pal.size() <= 256;
  const int depth = !palette ? 8 : pal.size() <= 2 ? 1 : pal.size() <= 4 ? 2 : pal.size() <= 16 ? 4 : 8;
  const size_t stride = palette ? 1 + (W * (size_t)depth + 7) / 8 : 1 + 4 * W;
  std::vector<uint8_t> rows(stride * H, 0);
  auto convert = [&](int t) {
    size_t y0, y1;
    rows_of(t, y0, y1);
    for (size_t y = y0; y < y1; y++) {
      uint8_t *out = rows.data() + y * stride;
      const uint8_t *in = rgba + 4 * W * y;
      out[0] = 0;  // filter: none
      if (!palette) {
        memcpy(out + 1, in, 4 * W);
        continue;
      }
      for (size_t x = 0; x < W; x++) {
        uint32_t c;
        memcpy(&c, in + 4 * x, 4);
        const uint32_t idx = (uint32_t)(std::lower_bound(pal.begin(), pal.end(), c) - pal.begin());
        const size_t bit = x * (size_t)depth;
        out[1 + bit / 8] |= (uint8_t)(idx << (8 - depth - (int)(bit % 8)));
      }
    }
  };
  {
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; t++) pool.emplace_back(convert, t);
    convert(0);
    for (auto &th : pool) th.join();
  }
  // palette entries as 0xAABBGGRR: the bytes R, G, B, A of the pixel in memory order
  std::vector<uint32_t> pal_abgr(pal.size());
  for (size_t i = 0; i < pal.size(); i++) {
    const uint8_t *b = (const uint8_t *)&pal[i];
    pal_abgr[i] = (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
  }
  const int rc = phde_png_write_rows(path, rows.data(), width, height, depth, palette ? 3 : 6, pal_abgr.data(),
                                     (int)pal_abgr.size(), nthreads);
  return rc == 0 ? PHDE_OK : PHDE_ERR_INVALID;
}
