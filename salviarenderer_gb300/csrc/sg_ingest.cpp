// sg_ingest.cpp -- host side of texture and mesh ingest for the drop-in API:
// a PNG decoder on its own inflate, PNG and Radiance RGBE writers on its own
// deflate, and the Wavefront OBJ / MTL loader of create_mesh_from_obj.
//
// Reference: salvia/src/ext/resource/texture/tex_io.cpp (load_texture,
// load_cube, save_surface -- FreeImage decodes and encodes there; it is not
// part of the reference's sources) and salvia/src/ext/resource/mesh/
// mesh_io_obj.cpp (load_obj_mesh_c, load_material, construct_meshes).  The
// format tables below (DEFLATE's length / distance bases, the code-length
// order, PNG's chunk layout, Adam7's pass grid) are the published formats'
// own (RFC 1950, RFC 1951, the PNG specification, Ward's RGBE).
//
// The device half (pixel-format conversion into a texture level, and back
// out of one for saving) is in sg_api.cu / sg_misc.cu.
#include "sg_ingest.h"

#include <algorithm>
#include <cerrno>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iterator>
#include <memory>
#include <string>
#include <unordered_map>

#include "salvia_gb300.h"

namespace sg::ingest {
namespace {

// ---- checksums --------------------------------------------------------------

struct Crc32Table {
  uint32_t t[256];
  Crc32Table() {
    for (uint32_t n = 0; n < 256; ++n) {
      uint32_t c = n;
      for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      t[n] = c;
    }
  }
};
// CRC-32 of PNG chunks (ISO 3309 polynomial, reflected)
uint32_t crc32(uint8_t const* p, size_t n) {
  static Crc32Table const tab;
  uint32_t c = 0xFFFFFFFFu;
  for (size_t i = 0; i < n; ++i) c = tab.t[(c ^ p[i]) & 0xFFu] ^ (c >> 8);
  return c ^ 0xFFFFFFFFu;
}
// Adler-32 of the zlib trailer (RFC 1950 section 8)
uint32_t adler32(uint8_t const* p, size_t n) {
  uint32_t s1 = 1, s2 = 0;
  while (n) {
    size_t k = std::min<size_t>(n, 5552);  // the largest run whose sums fit 32 bits
    n -= k;
    while (k--) {
      s1 += *p++;
      s2 += s1;
    }
    s1 %= 65521u;
    s2 %= 65521u;
  }
  return (s2 << 16) | s1;
}

uint32_t be32(uint8_t const* p) {
  return (uint32_t(p[0]) << 24) | (uint32_t(p[1]) << 16) | (uint32_t(p[2]) << 8) | uint32_t(p[3]);
}
void put_be32(std::vector<uint8_t>& o, uint32_t v) {
  o.push_back(uint8_t(v >> 24));
  o.push_back(uint8_t(v >> 16));
  o.push_back(uint8_t(v >> 8));
  o.push_back(uint8_t(v));
}
uint32_t reverse_bits(uint32_t v, int n) {
  uint32_t r = 0;
  for (int i = 0; i < n; ++i) r |= ((v >> i) & 1u) << (n - 1 - i);
  return r;
}

// ---- DEFLATE tables (RFC 1951 section 3.2.5 and 3.2.7) ----------------------

constexpr uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                   31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
constexpr uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
constexpr uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                    193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
constexpr uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
constexpr uint8_t kCodeLenOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

// LSB-first bit reader over a byte range.
class BitReader {
 public:
  BitReader(uint8_t const* p, size_t n) : p_(p), n_(n) {}
  void top_up() {
    while (cnt_ <= 56 && pos_ < n_) {
      buf_ |= static_cast<uint64_t>(p_[pos_++]) << cnt_;
      cnt_ += 8;
    }
  }
  int avail() const { return cnt_; }
  uint32_t peek(int k) const { return static_cast<uint32_t>(buf_ & ((uint64_t(1) << k) - 1)); }
  void drop(int k) {
    buf_ >>= k;
    cnt_ -= k;
  }
  bool get(int k, uint32_t& v) {
    if (cnt_ < k) top_up();
    if (cnt_ < k) return false;
    v = peek(k);
    drop(k);
    return true;
  }
  void to_byte() { drop(cnt_ & 7); }
  bool copy_bytes(uint8_t* dst, size_t len) {
    while (len && cnt_ >= 8) {
      *dst++ = static_cast<uint8_t>(buf_);
      drop(8);
      --len;
    }
    if (n_ - pos_ < len) return false;
    std::memcpy(dst, p_ + pos_, len);
    pos_ += len;
    return true;
  }

 private:
  uint8_t const* p_;
  size_t n_, pos_ = 0;
  uint64_t buf_ = 0;
  int cnt_ = 0;
};

// A canonical Huffman code (RFC 1951 section 3.2.2): a table on the next
// kFast bits for the short codes, a bit-serial walk of the canonical order
// for the rest.
struct Huffman {
  static constexpr int kFast = 10;
  uint16_t fast[1 << kFast];  // symbol << 4 | length; 0 = longer or unused code
  uint16_t count[16];
  uint16_t sym[320];

  // false for an over-subscribed code, and for an incomplete one unless
  // `lone_ok` and it is a single one-bit code (or empty)
  bool build(uint8_t const* len, int n, bool lone_ok) {
    std::memset(count, 0, sizeof count);
    for (int i = 0; i < n; ++i) ++count[len[i]];
    count[0] = 0;
    int left = 1, maxlen = 0;
    for (int l = 1; l < 16; ++l) {
      left = (left << 1) - count[l];
      if (left < 0) return false;
      if (count[l]) maxlen = l;
    }
    if (left > 0 && (!lone_ok || maxlen > 1)) return false;
    uint16_t offs[16];
    offs[1] = 0;
    for (int l = 1; l < 15; ++l) offs[l + 1] = static_cast<uint16_t>(offs[l] + count[l]);
    for (int i = 0; i < n; ++i)
      if (len[i]) sym[offs[len[i]]++] = static_cast<uint16_t>(i);
    std::memset(fast, 0, sizeof fast);
    uint32_t code = 0;
    int k = 0;
    for (int l = 1; l <= 15; ++l) {
      for (int j = 0; j < count[l]; ++j, ++k, ++code) {
        if (l > kFast) continue;
        uint32_t const r = reverse_bits(code, l);
        for (uint32_t x = r; x < (1u << kFast); x += 1u << l) fast[x] = static_cast<uint16_t>(sym[k] << 4 | l);
      }
      code <<= 1;
    }
    return true;
  }
  // the next symbol, or -1
  int decode(BitReader& br) const {
    br.top_up();
    int const avail = br.avail();
    if (avail >= kFast) {
      uint16_t const e = fast[br.peek(kFast)];
      if (e) {
        br.drop(e & 15);
        return e >> 4;
      }
    }
    uint32_t const bits = br.peek(std::min(avail, 15));
    int code = 0, first = 0, index = 0;
    for (int l = 1; l <= 15 && l <= avail; ++l) {
      code |= static_cast<int>((bits >> (l - 1)) & 1u);
      int const c = count[l];
      if (code - first < c) {
        br.drop(l);
        return sym[index + code - first];
      }
      index += c;
      first = (first + c) << 1;
      code <<= 1;
    }
    return -1;
  }
};

struct FixedCodes {
  Huffman lit, dist;
  FixedCodes() {
    uint8_t l[288];
    for (int i = 0; i < 288; ++i) l[i] = i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8;
    lit.build(l, 288, false);
    uint8_t d[32];
    std::fill(d, d + 32, uint8_t(5));  // 30 and 31 complete the code; never valid in a stream
    dist.build(d, 32, false);
  }
};

bool read_dynamic(BitReader& br, Huffman& lit, Huffman& dist) {
  uint32_t hlit, hdist, hclen;
  if (!br.get(5, hlit) || !br.get(5, hdist) || !br.get(4, hclen)) return false;
  hlit += 257;
  hdist += 1;
  hclen += 4;
  if (hlit > 286 || hdist > 30) return false;
  uint8_t cl[19] = {};
  for (uint32_t i = 0; i < hclen; ++i) {
    uint32_t v;
    if (!br.get(3, v)) return false;
    cl[kCodeLenOrder[i]] = static_cast<uint8_t>(v);
  }
  Huffman clh;
  if (!clh.build(cl, 19, false)) return false;
  uint8_t lens[320] = {};
  uint32_t const total = hlit + hdist;
  uint32_t idx = 0;
  while (idx < total) {
    int const s = clh.decode(br);
    if (s < 0) return false;
    if (s < 16) {
      lens[idx++] = static_cast<uint8_t>(s);
      continue;
    }
    uint32_t rep, extra;
    uint8_t val = 0;
    if (s == 16) {
      if (idx == 0 || !br.get(2, extra)) return false;
      val = lens[idx - 1];
      rep = 3 + extra;
    } else if (s == 17) {
      if (!br.get(3, extra)) return false;
      rep = 3 + extra;
    } else {
      if (!br.get(7, extra)) return false;
      rep = 11 + extra;
    }
    if (idx + rep > total) return false;
    while (rep--) lens[idx++] = val;
  }
  if (lens[256] == 0) return false;  // no end-of-block code
  return lit.build(lens, static_cast<int>(hlit), true) && dist.build(lens + hlit, static_cast<int>(hdist), true);
}

// Raw DEFLATE into out[0, out.size()); `produced` = bytes written.
bool inflate_raw(BitReader& br, std::vector<uint8_t>& out, size_t& produced) {
  static FixedCodes const fixed;
  auto dyn = std::make_unique<Huffman[]>(2);
  uint8_t* const o = out.data();
  size_t const cap = out.size();
  size_t n = 0;
  for (;;) {
    uint32_t final, type;
    if (!br.get(1, final) || !br.get(2, type)) return false;
    if (type == 0) {
      br.to_byte();
      uint32_t len, nlen;
      if (!br.get(16, len) || !br.get(16, nlen) || (len ^ 0xFFFFu) != nlen) return false;
      if (cap - n < len || !br.copy_bytes(o + n, len)) return false;
      n += len;
    } else if (type == 3) {
      return false;
    } else {
      Huffman const* lit = &fixed.lit;
      Huffman const* dist = &fixed.dist;
      if (type == 2) {
        if (!read_dynamic(br, dyn[0], dyn[1])) return false;
        lit = &dyn[0];
        dist = &dyn[1];
      }
      for (;;) {
        int s = lit->decode(br);
        if (s < 0) return false;
        if (s < 256) {
          if (n >= cap) return false;
          o[n++] = static_cast<uint8_t>(s);
          continue;
        }
        if (s == 256) break;
        s -= 257;
        if (s >= 29) return false;
        uint32_t e;
        if (!br.get(kLenExtra[s], e)) return false;
        size_t const len = kLenBase[s] + e;
        int const d = dist->decode(br);
        if (d < 0 || d >= 30 || !br.get(kDistExtra[d], e)) return false;
        size_t const back = kDistBase[d] + e;
        if (back > n || cap - n < len) return false;
        uint8_t* w = o + n;
        uint8_t const* r = w - back;
        for (size_t i = 0; i < len; ++i) w[i] = r[i];  // overlapping copies repeat the run
        n += len;
      }
    }
    if (final) break;
  }
  produced = n;
  return true;
}

// LSB-first bit writer.
class BitWriter {
 public:
  explicit BitWriter(std::vector<uint8_t>& o) : o_(o) {}
  void put(uint32_t v, int k) {
    buf_ |= static_cast<uint64_t>(v) << cnt_;
    cnt_ += k;
    while (cnt_ >= 8) {
      o_.push_back(static_cast<uint8_t>(buf_));
      buf_ >>= 8;
      cnt_ -= 8;
    }
  }
  void put_code(uint32_t code, int len) { put(reverse_bits(code, len), len); }  // Huffman codes go MSB first
  void flush() {
    if (cnt_ > 0) o_.push_back(static_cast<uint8_t>(buf_));
    buf_ = 0;
    cnt_ = 0;
  }

 private:
  std::vector<uint8_t>& o_;
  uint64_t buf_ = 0;
  int cnt_ = 0;
};

void put_fixed_literal(BitWriter& bw, int s) {
  if (s < 144) bw.put_code(0x30u + s, 8);
  else if (s < 256) bw.put_code(0x190u + (s - 144), 9);
  else if (s < 280) bw.put_code(static_cast<uint32_t>(s - 256), 7);
  else bw.put_code(0xC0u + (s - 280), 8);
}

bool is_c_space(int c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }

}  // namespace

bool zlib_inflate(uint8_t const* src, size_t n, std::vector<uint8_t>& out) {
  if (n < 6) return false;
  uint32_t const cmf = src[0], flg = src[1];
  if ((cmf & 15u) != 8u || (cmf >> 4) > 7u || ((cmf << 8) | flg) % 31u != 0u || (flg & 0x20u)) return false;
  BitReader br(src + 2, n - 2);
  size_t produced = 0;
  if (!inflate_raw(br, out, produced) || produced != out.size()) return false;
  br.to_byte();
  uint32_t a = 0;
  for (int i = 0; i < 4; ++i) {
    uint32_t b;
    if (!br.get(8, b)) return false;
    a = (a << 8) | b;
  }
  return a == adler32(out.data(), out.size());
}

// LZ77 over a 32 KB window (hash chains on 3-byte prefixes, at most 64
// candidates) coded with DEFLATE's fixed Huffman codes in one block.
std::vector<uint8_t> zlib_deflate(uint8_t const* src, size_t n) {
  std::vector<uint8_t> o;
  o.reserve(n / 2 + 64);
  o.push_back(0x78);  // deflate, 32 KB window
  o.push_back(0x01);  // (0x7801 % 31 == 0), no dictionary
  BitWriter bw(o);
  bw.put(1, 1);  // final block
  bw.put(1, 2);  // fixed codes
  constexpr size_t kWin = 32768, kMask = kWin - 1;
  constexpr int kChain = 64;
  std::vector<int64_t> head(1u << 15, -1), prev(kWin, -1);
  auto hash = [&](size_t p) {
    return ((uint32_t(src[p]) << 10) ^ (uint32_t(src[p + 1]) << 5) ^ uint32_t(src[p + 2])) & 0x7FFFu;
  };
  auto insert = [&](size_t p) {
    if (p + 2 >= n) return;
    uint32_t const h = hash(p);
    prev[p & kMask] = head[h];
    head[h] = static_cast<int64_t>(p);
  };
  size_t i = 0;
  while (i < n) {
    size_t best = 0, best_d = 0;
    if (i + 2 < n) {
      int64_t cand = head[hash(i)];
      size_t const lim = std::min<size_t>(258, n - i);
      for (int c = 0; cand >= 0 && c < kChain; ++c) {
        size_t const cp = static_cast<size_t>(cand);
        if (i - cp > kWin) break;
        size_t l = 0;
        while (l < lim && src[cp + l] == src[i + l]) ++l;
        if (l > best) {
          best = l;
          best_d = i - cp;
          if (l == lim) break;
        }
        int64_t const nx = prev[cp & kMask];
        if (nx >= cand) break;  // the slot was reused by a later position
        cand = nx;
      }
    }
    if (best >= 3) {
      int s = 28;
      while (kLenBase[s] > best) --s;
      put_fixed_literal(bw, 257 + s);
      bw.put(static_cast<uint32_t>(best - kLenBase[s]), kLenExtra[s]);
      int d = 29;
      while (kDistBase[d] > best_d) --d;
      bw.put_code(static_cast<uint32_t>(d), 5);
      bw.put(static_cast<uint32_t>(best_d - kDistBase[d]), kDistExtra[d]);
      for (size_t k = 0; k < best; ++k) insert(i + k);
      i += best;
    } else {
      put_fixed_literal(bw, src[i]);
      insert(i);
      ++i;
    }
  }
  put_fixed_literal(bw, 256);
  bw.flush();
  put_be32(o, adler32(src, n));
  return o;
}

// ---- PNG --------------------------------------------------------------------

namespace {
struct PassGrid {
  uint32_t x0, y0, dx, dy;
};
constexpr PassGrid kAdam7[7] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4},
                                {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};

int paeth(int a, int b, int c) {
  int const p = a + b - c;
  int const pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
  if (pa <= pb && pa <= pc) return a;
  return pb <= pc ? b : c;
}

// Reverses one scanline's filter in place; `prev` is the unfiltered line
// above (nullptr for the first line of a pass).
bool unfilter(uint8_t ft, uint8_t* cur, uint8_t const* prev, size_t len, size_t bpp) {
  switch (ft) {
  case 0: return true;
  case 1:
    for (size_t i = bpp; i < len; ++i) cur[i] = static_cast<uint8_t>(cur[i] + cur[i - bpp]);
    return true;
  case 2:
    if (prev)
      for (size_t i = 0; i < len; ++i) cur[i] = static_cast<uint8_t>(cur[i] + prev[i]);
    return true;
  case 3:
    for (size_t i = 0; i < len; ++i) {
      int const a = i >= bpp ? cur[i - bpp] : 0, b = prev ? prev[i] : 0;
      cur[i] = static_cast<uint8_t>(cur[i] + ((a + b) >> 1));
    }
    return true;
  case 4:
    for (size_t i = 0; i < len; ++i) {
      int const a = i >= bpp ? cur[i - bpp] : 0, b = prev ? prev[i] : 0;
      int const c = (prev && i >= bpp) ? prev[i - bpp] : 0;
      cur[i] = static_cast<uint8_t>(cur[i] + paeth(a, b, c));
    }
    return true;
  default: return false;
  }
}

bool chunk_is(uint8_t const* t, char const* name) { return std::memcmp(t, name, 4) == 0; }
}  // namespace

int32_t decode_png(uint8_t const* p, size_t n, Image& out) {
  static uint8_t const kSig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
  if (!p || n < 8 || std::memcmp(p, kSig, 8) != 0) return SG_FAILED;
  size_t pos = 8;
  bool have_ihdr = false, have_iend = false, in_idat = false, idat_done = false, trns = false;
  uint32_t w = 0, h = 0;
  uint8_t depth = 0, ctype = 0, interlace = 0;
  std::vector<uint8_t> z;
  while (pos + 12 <= n) {
    uint32_t const len = be32(p + pos);
    if (len > 0x7FFFFFFFu || n - pos - 12 < len) return SG_FAILED;
    uint8_t const* type = p + pos + 4;
    uint8_t const* data = type + 4;
    bool const critical = !(type[0] & 0x20);
    pos += 12 + static_cast<size_t>(len);
    if (crc32(type, static_cast<size_t>(len) + 4) != be32(data + len)) {
      if (critical) return SG_FAILED;
      continue;  // a damaged ancillary chunk is dropped
    }
    if (!have_ihdr && !chunk_is(type, "IHDR")) return SG_FAILED;
    if (chunk_is(type, "IDAT")) {
      if (idat_done) return SG_FAILED;  // image data must be one run of chunks
      in_idat = true;
      z.insert(z.end(), data, data + len);
      continue;
    }
    if (in_idat) idat_done = true;
    if (chunk_is(type, "IHDR")) {
      if (have_ihdr || len != 13) return SG_FAILED;
      have_ihdr = true;
      w = be32(data);
      h = be32(data + 4);
      depth = data[8];
      ctype = data[9];
      interlace = data[12];
      if (w == 0 || h == 0 || w > 0x7FFFFFFFu || h > 0x7FFFFFFFu) return SG_FAILED;
      if (data[10] != 0 || data[11] != 0 || interlace > 1) return SG_FAILED;
    } else if (chunk_is(type, "IEND")) {
      have_iend = true;
      break;
    } else if (chunk_is(type, "tRNS")) {
      trns = true;
    } else if (critical && !chunk_is(type, "PLTE")) {
      return SG_FAILED;  // an unknown critical chunk
    }
  }
  if (!have_ihdr || !have_iend || z.empty()) return SG_FAILED;
  // the bitmaps copy_image_to_surface takes: 8-bit RGB and RGBA
  if (depth != 8 || (ctype != 2 && ctype != 6)) return SG_FAILED;
  if (ctype == 2 && trns) return SG_FAILED;  // a keyed colour would need an alpha channel
  uint32_t const ch = ctype == 6 ? 4u : 3u;
  if (static_cast<uint64_t>(w) * h > (uint64_t(1) << 28)) return SG_FAILED;
  // the filtered scanlines of every pass, each with its filter byte
  uint64_t total = 0;
  int const npass = interlace ? 7 : 1;
  uint32_t pw[7], ph[7];
  for (int k = 0; k < npass; ++k) {
    PassGrid const g = interlace ? kAdam7[k] : PassGrid{0, 0, 1, 1};
    pw[k] = w > g.x0 ? (w - g.x0 + g.dx - 1) / g.dx : 0;
    ph[k] = h > g.y0 ? (h - g.y0 + g.dy - 1) / g.dy : 0;
    if (pw[k] && ph[k]) total += static_cast<uint64_t>(ph[k]) * (1 + static_cast<uint64_t>(pw[k]) * ch);
  }
  std::vector<uint8_t> raw(static_cast<size_t>(total));
  if (!zlib_inflate(z.data(), z.size(), raw)) return SG_FAILED;
  out.w = w;
  out.h = h;
  out.channels = ch;
  out.px.assign(static_cast<size_t>(w) * h * ch, 0);
  uint8_t* f = raw.data();
  for (int k = 0; k < npass; ++k) {
    if (!pw[k] || !ph[k]) continue;
    PassGrid const g = interlace ? kAdam7[k] : PassGrid{0, 0, 1, 1};
    size_t const rowlen = static_cast<size_t>(pw[k]) * ch;
    uint8_t const* prev = nullptr;
    for (uint32_t r = 0; r < ph[k]; ++r) {
      uint8_t* cur = f + 1;
      if (!unfilter(f[0], cur, prev, rowlen, ch)) return SG_FAILED;
      uint32_t const y = g.y0 + r * g.dy;
      uint8_t* dst_row = out.px.data() + static_cast<size_t>(h - 1 - y) * w * ch;  // FreeImage keeps rows bottom-up
      if (!interlace) {
        std::memcpy(dst_row, cur, rowlen);
      } else {
        for (uint32_t c = 0; c < pw[k]; ++c)
          std::memcpy(dst_row + static_cast<size_t>(g.x0 + c * g.dx) * ch, cur + static_cast<size_t>(c) * ch, ch);
      }
      prev = cur;
      f += 1 + rowlen;
    }
  }
  return SG_OK;
}

namespace {
void put_chunk(std::vector<uint8_t>& o, char const* type, uint8_t const* data, size_t len) {
  put_be32(o, static_cast<uint32_t>(len));
  size_t const at = o.size();
  o.insert(o.end(), type, type + 4);
  if (len) o.insert(o.end(), data, data + len);
  put_be32(o, crc32(o.data() + at, len + 4));
}
}  // namespace

std::vector<uint8_t> encode_png(uint8_t const* px, uint32_t w, uint32_t h, uint32_t ch) {
  size_t const rowlen = static_cast<size_t>(w) * ch;
  std::vector<uint8_t> raw;
  raw.reserve((rowlen + 1) * h);
  std::vector<uint8_t> cand[5];
  for (auto& c : cand) c.resize(rowlen);
  for (uint32_t r = 0; r < h; ++r) {
    uint8_t const* cur = px + static_cast<size_t>(h - 1 - r) * rowlen;  // the file's top line is the last row
    uint8_t const* up = r ? px + static_cast<size_t>(h - r) * rowlen : nullptr;
    // each filter, then the one with the smallest sum of |signed byte|
    uint64_t best_cost = UINT64_MAX;
    int best = 0;
    for (int ft = 0; ft < 5; ++ft) {
      uint64_t cost = 0;
      for (size_t i = 0; i < rowlen; ++i) {
        int const a = i >= ch ? cur[i - ch] : 0, b = up ? up[i] : 0, c = (up && i >= ch) ? up[i - ch] : 0;
        int const pred = ft == 0 ? 0 : ft == 1 ? a : ft == 2 ? b : ft == 3 ? (a + b) >> 1 : paeth(a, b, c);
        uint8_t const v = static_cast<uint8_t>(cur[i] - pred);
        cand[ft][i] = v;
        cost += static_cast<uint64_t>(std::abs(static_cast<int>(static_cast<int8_t>(v))));
      }
      if (cost < best_cost) {
        best_cost = cost;
        best = ft;
      }
    }
    raw.push_back(static_cast<uint8_t>(best));
    raw.insert(raw.end(), cand[best].begin(), cand[best].end());
  }
  std::vector<uint8_t> const z = zlib_deflate(raw.data(), raw.size());
  std::vector<uint8_t> o = {137, 80, 78, 71, 13, 10, 26, 10};
  uint8_t ihdr[13];
  uint32_t const dims[2] = {w, h};
  for (int k = 0; k < 2; ++k)
    for (int b = 0; b < 4; ++b) ihdr[k * 4 + b] = static_cast<uint8_t>(dims[k] >> (24 - 8 * b));
  ihdr[8] = 8;
  ihdr[9] = ch == 4 ? 6 : 2;
  ihdr[10] = ihdr[11] = ihdr[12] = 0;
  put_chunk(o, "IHDR", ihdr, 13);
  constexpr size_t kIdat = size_t(1) << 20;
  for (size_t at = 0; at < z.size(); at += kIdat) put_chunk(o, "IDAT", z.data() + at, std::min(kIdat, z.size() - at));
  put_chunk(o, "IEND", nullptr, 0);
  return o;
}

// ---- Radiance RGBE ----------------------------------------------------------

namespace {
// Ward's float -> RGBE: the shared exponent of the largest component, each
// mantissa truncated to 8 bits.  Negative and non-finite components write 0;
// a mantissa that rounds to 256 is held at 255.
void float_to_rgbe(float r, float g, float b, uint8_t* o) {
  auto clean = [](float v) { return (std::isfinite(v) && v > 0.0f) ? v : 0.0f; };
  r = clean(r);
  g = clean(g);
  b = clean(b);
  float const v = std::max(r, std::max(g, b));
  if (v < 1e-32f) {
    o[0] = o[1] = o[2] = o[3] = 0;
    return;
  }
  int e = 0;
  float const m = std::frexp(v, &e) * 256.0f / v;
  auto q = [&](float c) { return static_cast<uint8_t>(std::min(255.0f, c * m)); };
  o[0] = q(r);
  o[1] = q(g);
  o[2] = q(b);
  o[3] = static_cast<uint8_t>(e + 128);
}
// one channel of a scanline, run-length coded: runs of 4+ equal bytes as
// (128 + n, byte), the rest as (n, n bytes)
void rle_channel(std::vector<uint8_t>& o, uint8_t const* b, size_t w) {
  size_t i = 0;
  while (i < w) {
    size_t run_at = i, run = 0;
    while (run_at < w) {
      run = 1;
      while (run_at + run < w && run < 127 && b[run_at + run] == b[run_at]) ++run;
      if (run >= 4) break;
      run_at += run;
    }
    if (run < 4) run_at = w;
    while (i < run_at) {
      size_t const k = std::min<size_t>(128, run_at - i);
      o.push_back(static_cast<uint8_t>(k));
      o.insert(o.end(), b + i, b + i + k);
      i += k;
    }
    if (run_at < w) {
      o.push_back(static_cast<uint8_t>(128 + run));
      o.push_back(b[run_at]);
      i = run_at + run;
    }
  }
}
}  // namespace

std::vector<uint8_t> encode_hdr(float const* rgb, uint32_t w, uint32_t h) {
  std::string head = "#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y " + std::to_string(h) + " +X " + std::to_string(w) + "\n";
  std::vector<uint8_t> o(head.begin(), head.end());
  bool const rle = w >= 8 && w <= 0x7FFF;
  std::vector<uint8_t> line(static_cast<size_t>(w) * 4), chan(w);
  for (uint32_t r = 0; r < h; ++r) {
    float const* src = rgb + static_cast<size_t>(h - 1 - r) * w * 3;  // the file's top line is the last row
    for (uint32_t x = 0; x < w; ++x) float_to_rgbe(src[x * 3], src[x * 3 + 1], src[x * 3 + 2], &line[x * 4]);
    if (!rle) {
      o.insert(o.end(), line.begin(), line.end());
      continue;
    }
    o.push_back(2);
    o.push_back(2);
    o.push_back(static_cast<uint8_t>(w >> 8));
    o.push_back(static_cast<uint8_t>(w & 0xFF));
    for (int c = 0; c < 4; ++c) {
      for (uint32_t x = 0; x < w; ++x) chan[x] = line[x * 4 + c];
      rle_channel(o, chan.data(), w);
    }
  }
  return o;
}

// ---- Wavefront OBJ / MTL ----------------------------------------------------

namespace {

constexpr size_t kTokenMax = 2047;  // the reference reads tokens into 2048-byte buffers

// The file as load_obj_mesh_c reads it: a stdio stream under fscanf("%s"),
// fscanf("%f"), fscanf("%u"), fgetc and ungetc (end-of-file indicator
// included).  Numbers: the longest prefix strtof / strtoul accept.
class CStream {
 public:
  explicit CStream(std::string s) : s_(std::move(s)) {}
  int get() {
    if (pos_ >= s_.size()) {
      eof_ = true;
      return -1;
    }
    return static_cast<unsigned char>(s_[pos_++]);
  }
  void unget(int c) {
    if (c >= 0) --pos_;
  }
  int peek() {
    int const c = get();
    unget(c);
    return c;
  }
  bool eof() const { return eof_; }
  bool skip_space() {
    for (;;) {
      int const c = get();
      if (c < 0) return false;
      if (!is_c_space(c)) {
        unget(c);
        return true;
      }
    }
  }
  // %s: 1 with a token, -1 at the end of the file; `too_long` past the buffer
  int token(std::string& t, bool& too_long) {
    if (!skip_space()) return -1;
    t.clear();
    for (;;) {
      int const c = get();
      if (c < 0) break;
      if (is_c_space(c)) {
        unget(c);
        break;
      }
      t.push_back(static_cast<char>(c));
    }
    if (t.size() > kTokenMax) too_long = true;
    return 1;
  }
  int scan_float(float& v) {
    if (!skip_space()) return -1;
    char const* b = s_.c_str() + pos_;
    char* e = nullptr;
    float const f = std::strtof(b, &e);
    if (e == b) return 0;
    pos_ += static_cast<size_t>(e - b);
    v = f;
    return 1;
  }
  int scan_uint(uint32_t& v) {
    if (!skip_space()) return -1;
    size_t q = pos_;
    bool neg = false;
    if (q < s_.size() && (s_[q] == '+' || s_[q] == '-')) neg = s_[q++] == '-';
    size_t const d0 = q;
    unsigned long long acc = 0;
    bool over = false;
    while (q < s_.size() && s_[q] >= '0' && s_[q] <= '9') {
      unsigned const dig = static_cast<unsigned>(s_[q] - '0');
      if (acc > (ULLONG_MAX - dig) / 10) over = true;
      acc = acc * 10 + dig;
      ++q;
    }
    if (q == d0) return 0;
    pos_ = q;
    if (over) acc = ULLONG_MAX;
    if (neg && !over) acc = 0ull - acc;
    v = static_cast<uint32_t>(acc);
    return 1;
  }
  // ignore(f, max_count, delim) (mesh_io_obj.cpp:53-61)
  void ignore(int max_count, int delim) {
    int cur = 0;
    while (!eof_ && cur++ < max_count) {
      int const ch = get();
      if (ch == delim) break;
    }
  }

 private:
  std::string s_;
  size_t pos_ = 0;
  bool eof_ = false;
};

// The material library as load_material reads it: std::istream extraction
// (operator>> for strings, float and int, ignore) with the stream's
// fail / end-of-file states.
class CxxStream {
 public:
  explicit CxxStream(std::string s) : s_(std::move(s)) {}
  bool ok() const { return !fail_; }
  bool read(std::string& t) {
    if (!sentry()) return false;
    t.clear();
    while (pos_ < s_.size() && !is_c_space(static_cast<unsigned char>(s_[pos_]))) t.push_back(s_[pos_++]);
    if (pos_ >= s_.size()) eof_ = true;
    return true;
  }
  // num_get for float: sign, digits, one point, exponent; the whole run must
  // convert, else 0 and fail; an infinite result is FLT_MAX and fail
  bool read(float& v) {
    if (!sentry()) return false;
    std::string acc;
    size_t q = pos_;
    auto at = [&](size_t i) { return i < s_.size() ? s_[i] : '\0'; };
    if (at(q) == '+' || at(q) == '-') acc.push_back(s_[q++]);
    bool digits = false, point = false;
    for (;;) {
      char const c = at(q);
      if (c >= '0' && c <= '9') {
        digits = true;
      } else if (c == '.' && !point) {
        point = true;
      } else {
        break;
      }
      acc.push_back(c);
      ++q;
    }
    if (digits && (at(q) == 'e' || at(q) == 'E')) {
      acc.push_back(s_[q++]);
      if (at(q) == '+' || at(q) == '-') acc.push_back(s_[q++]);
      while (at(q) >= '0' && at(q) <= '9') acc.push_back(s_[q++]);
    }
    pos_ = q;
    if (pos_ >= s_.size()) eof_ = true;
    char* e = nullptr;
    float const f = std::strtof(acc.c_str(), &e);
    if (acc.empty() || *e != '\0') {
      v = 0.0f;
      fail_ = true;
      return false;
    }
    if (std::isinf(f)) {
      v = f > 0 ? FLT_MAX : -FLT_MAX;
      fail_ = true;
      return false;
    }
    v = f;
    return true;
  }
  bool read(int& v) {
    if (!sentry()) return false;
    std::string acc;
    size_t q = pos_;
    if (q < s_.size() && (s_[q] == '+' || s_[q] == '-')) acc.push_back(s_[q++]);
    while (q < s_.size() && s_[q] >= '0' && s_[q] <= '9') acc.push_back(s_[q++]);
    pos_ = q;
    if (pos_ >= s_.size()) eof_ = true;
    if (acc.empty() || acc == "+" || acc == "-") {
      v = 0;
      fail_ = true;
      return false;
    }
    errno = 0;
    long long const l = std::strtoll(acc.c_str(), nullptr, 10);
    if (errno == ERANGE || l > INT_MAX || l < INT_MIN) {
      v = l > 0 ? INT_MAX : INT_MIN;
      fail_ = true;
      return false;
    }
    v = static_cast<int>(l);
    return true;
  }
  void ignore(size_t n, char delim) {
    if (fail_ || eof_) {
      fail_ = true;
      return;
    }
    for (size_t i = 0; i < n; ++i) {
      if (pos_ >= s_.size()) {
        eof_ = true;
        return;
      }
      if (s_[pos_++] == delim) return;
    }
  }

 private:
  bool sentry() {
    if (fail_ || eof_) {
      fail_ = true;
      return false;
    }
    while (pos_ < s_.size() && is_c_space(static_cast<unsigned char>(s_[pos_]))) ++pos_;
    if (pos_ >= s_.size()) {
      eof_ = true;
      fail_ = true;
      return false;
    }
    return true;
  }
  std::string s_;
  size_t pos_ = 0;
  bool fail_ = false, eof_ = false;
};

// obj_material (material.h, material.cpp:4-13)
struct Material {
  std::string name = "default";
  float ambient[4] = {0.2f, 0.2f, 0.2f, 1.0f};
  float diffuse[4] = {0.5f, 0.5f, 0.5f, 1.0f};
  float specular[4] = {0.7f, 0.7f, 0.7f, 1.0f};
  int shininess = 2;
  float alpha = 1.0f;
  bool is_specular = true;
  std::string tex_name, tex_path;
};

struct ObjVertex {
  float v[12];  // pos, uv, normal (obj_mesh_vertex, mesh_io_obj.cpp:41-45)
};

struct Triple {
  uint32_t p, t, n;
  bool operator==(Triple const& o) const { return p == o.p && t == o.t && n == o.n; }
};
struct TripleHasher {
  size_t operator()(Triple const& k) const {
    uint64_t h = (uint64_t(k.p) * 0x9E3779B97F4A7C15ull) ^ (uint64_t(k.t) * 0xC2B2AE3D27D4EB4Full) ^
                 (uint64_t(k.n) * 0x165667B19E3779F9ull);
    h ^= h >> 29;
    return static_cast<size_t>(h);
  }
};

bool read_file(std::string const& path, std::string& s) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  s.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
  return true;
}

// load_material (mesh_io_obj.cpp:59-138); false when the file cannot be read
bool load_material(std::vector<Material>& mtls, std::string const& text, std::filesystem::path const& base) {
  CxxStream in(text);
  Material* pm = nullptr;
  for (;;) {
    std::string cmd;
    in.read(cmd);
    if (!in.ok()) break;
    if (cmd == "#") {
      in.ignore(1000, '\n');
      continue;
    }
    if (cmd == "newmtl") {
      std::string nm;
      in.read(nm);
      for (auto& m : mtls)
        if (m.name == nm) {
          pm = &m;
          break;
        }
    }
    if (!pm) continue;
    auto rgb = [&](float* dst) {
      float c[3] = {0.0f, 0.0f, 0.0f};
      for (float& x : c)
        if (!in.read(x)) break;
      dst[0] = c[0];
      dst[1] = c[1];
      dst[2] = c[2];
      dst[3] = 0.0f;
    };
    if (cmd == "Ka") {
      rgb(pm->ambient);
    } else if (cmd == "Kd") {
      rgb(pm->diffuse);
    } else if (cmd == "Ks") {
      rgb(pm->specular);
    } else if (cmd == "d" || cmd == "Tr") {
      in.read(pm->alpha);
    } else if (cmd == "Ns") {
      in.read(pm->shininess);
    } else if (cmd == "illum") {
      int illum = 0;
      in.read(illum);
      pm->is_specular = illum == 2;
    } else if (cmd == "map_Kd") {
      in.read(pm->tex_name);
      std::replace(pm->tex_name.begin(), pm->tex_name.end(), '\\', '/');
      pm->tex_path = (base / pm->tex_name).generic_string();
    }
    in.ignore(1000, '\n');
  }
  return true;
}

struct ObjData {
  std::vector<ObjVertex> verts;
  std::vector<uint32_t> indices;
  std::vector<uint32_t> attrs;
  std::vector<Material> mtls;
};

// load_obj_mesh_c (mesh_io_obj.cpp:140-263)
int32_t load_obj(std::string const& fname, bool flip_tex_v, ObjData& r) {
  std::string text;
  if (!read_file(fname, text)) return SG_FAILED;
  CStream f(std::move(text));
  std::vector<float> positions, uvs, normals;  // 4 floats each
  r.mtls.emplace_back();
  uint32_t subset = 0;
  std::string mtl_fname;
  std::unordered_map<Triple, uint32_t, TripleHasher> smooth;
  bool too_long = false;
  std::string cmd, name;
  for (;;) {
    int const got = f.token(cmd, too_long);
    if (too_long) return SG_FAILED;
    if (got < 0 || f.eof()) break;
    if (cmd[0] == '#') {
      // comment
    } else if (cmd == "v" || cmd == "vn") {
      float x = 0.0f, y = 0.0f, z = 0.0f;
      if (f.scan_float(x) == 1 && f.scan_float(y) == 1) f.scan_float(z);
      float const w = cmd == "v" ? 1.0f : 0.0f;
      std::vector<float>& dst = cmd == "v" ? positions : normals;
      dst.insert(dst.end(), {x, y, z, w});
    } else if (cmd == "vt") {
      float u = 0.0f, v = 0.0f;
      if (f.scan_float(u) == 1) f.scan_float(v);
      uvs.insert(uvs.end(), {u, flip_tex_v ? 1.0f - v : v, 0.0f, 0.0f});
    } else if (cmd == "f") {
      uint32_t pi = 0, ti = 0, ni = 0;
      for (int corner = 0; corner < 3; ++corner) {
        ObjVertex vert{};
        f.scan_uint(pi);
        if (pi == 0 || pi > positions.size() / 4) return SG_FAILED;
        std::memcpy(vert.v, &positions[(pi - 1) * 4], 16);
        if (f.peek() == '/') {
          f.ignore(1, -1);
          if (f.peek() != '/') {
            f.scan_uint(ti);
            if (ti == 0 || ti > uvs.size() / 4) return SG_FAILED;
            std::memcpy(vert.v + 4, &uvs[(ti - 1) * 4], 16);
          }
          if (f.peek() == '/') {
            f.ignore(1, -1);
            f.scan_uint(ni);
            if (ni == 0 || ni > normals.size() / 4) return SG_FAILED;
            std::memcpy(vert.v + 8, &normals[(ni - 1) * 4], 16);
          }
        }
        // vertices are shared by index triple, the stale indices of the
        // face's earlier corners included (as the reference keys them)
        Triple const key{pi, ti, ni};
        auto it = smooth.find(key);
        uint32_t vi;
        if (it == smooth.end()) {
          vi = static_cast<uint32_t>(r.verts.size());
          smooth.emplace(key, vi);
          r.verts.push_back(vert);
        } else {
          vi = it->second;
        }
        r.indices.push_back(vi);
      }
      r.attrs.push_back(subset);
    } else if (cmd == "mtllib") {
      std::string t;
      if (f.token(t, too_long) == 1) mtl_fname = t;
      if (too_long) return SG_FAILED;
    } else if (cmd == "usemtl") {
      name.clear();
      f.token(name, too_long);
      if (too_long) return SG_FAILED;
      bool found = false;
      for (size_t i = 0; i < r.mtls.size(); ++i)
        if (r.mtls[i].name == name) {
          found = true;
          subset = static_cast<uint32_t>(i);
          break;
        }
      if (!found) {
        subset = static_cast<uint32_t>(r.mtls.size());
        r.mtls.emplace_back();
        r.mtls.back().name = name;
      }
    }
    f.ignore(65536, '\n');
  }
  std::filesystem::path const base = std::filesystem::absolute(std::filesystem::path(fname)).parent_path();
  if (!mtl_fname.empty()) {
    std::string mt;
    if (read_file((base / mtl_fname).string(), mt)) load_material(r.mtls, mt, base);
  }
  return SG_OK;
}

}  // namespace
}  // namespace sg::ingest

// ---- C ABI ------------------------------------------------------------------

namespace {
struct ObjStorage {
  std::vector<float> verts;
  std::vector<uint32_t> indices;
  std::vector<sg_obj_material> mats;
  std::vector<std::string> strings;
};
// standard layout: the sg_obj_mesh handed out is the holder's first member
struct ObjMeshHolder {
  sg_obj_mesh pub;
  ObjStorage* store;
};
int32_t to_blob(std::vector<uint8_t> const& v, sg_blob* out) {
  out->data = static_cast<uint8_t*>(std::malloc(v.empty() ? 1 : v.size()));
  if (!out->data) return SG_OUT_OF_MEMORY;
  if (!v.empty()) std::memcpy(out->data, v.data(), v.size());
  out->size = v.size();
  return SG_OK;
}
}  // namespace

extern "C" {

int32_t sg_image_decode(const void* file, size_t size, sg_image* out) try {
  if (!file || !out) return SG_INVALID_PARAMETER;
  *out = sg_image{};
  sg::ingest::Image img;
  if (int32_t r = sg::ingest::decode_png(static_cast<uint8_t const*>(file), size, img)) return r;
  out->pixels = static_cast<uint8_t*>(std::malloc(img.px.size()));
  if (!out->pixels) return SG_OUT_OF_MEMORY;
  std::memcpy(out->pixels, img.px.data(), img.px.size());
  out->width = img.w;
  out->height = img.h;
  out->channels = img.channels;
  return SG_OK;
} catch (std::bad_alloc const&) {
  return SG_OUT_OF_MEMORY;
}

void sg_image_release(sg_image* image) {
  if (!image) return;
  std::free(image->pixels);
  *image = sg_image{};
}

void sg_blob_release(sg_blob* blob) {
  if (!blob) return;
  std::free(blob->data);
  blob->data = nullptr;
  blob->size = 0;
}

int32_t sg_image_encode_png(const sg_image* image, sg_blob* out) try {
  if (!image || !out || !image->pixels || !image->width || !image->height ||
      (image->channels != 3 && image->channels != 4))
    return SG_INVALID_PARAMETER;
  *out = sg_blob{};
  return to_blob(sg::ingest::encode_png(image->pixels, image->width, image->height, image->channels), out);
} catch (std::bad_alloc const&) {
  return SG_OUT_OF_MEMORY;
}

int32_t sg_image_encode_hdr(const float* rgb, uint32_t width, uint32_t height, sg_blob* out) try {
  if (!rgb || !out || !width || !height) return SG_INVALID_PARAMETER;
  *out = sg_blob{};
  return to_blob(sg::ingest::encode_hdr(rgb, width, height), out);
} catch (std::bad_alloc const&) {
  return SG_OUT_OF_MEMORY;
}

int32_t sg_obj_load(const char* path, int32_t flip_tex_v, sg_obj_mesh** out) try {
  if (!path || !out) return SG_INVALID_PARAMETER;
  *out = nullptr;
  sg::ingest::ObjData d;
  if (int32_t r = sg::ingest::load_obj(path, flip_tex_v != 0, d)) return r;
  auto st = std::make_unique<ObjStorage>();
  st->verts.resize(d.verts.size() * 12);
  if (!d.verts.empty()) std::memcpy(st->verts.data(), d.verts.data(), d.verts.size() * sizeof(d.verts[0]));
  // construct_meshes (mesh_io_obj.cpp:375-434): a mesh per material with
  // faces, its indices in face order
  size_t const nm = d.mtls.size();
  std::vector<size_t> start(nm + 1, 0);
  for (uint32_t a : d.attrs) start[a + 1] += 3;
  for (size_t m = 0; m < nm; ++m) start[m + 1] += start[m];
  st->indices.resize(d.indices.size());
  std::vector<size_t> at(start.begin(), start.end() - 1);
  for (size_t i = 0; i < d.indices.size(); ++i) st->indices[at[d.attrs[i / 3]]++] = d.indices[i];
  std::vector<size_t> used;
  for (size_t m = 0; m < nm; ++m)
    if (start[m + 1] > start[m]) used.push_back(m);
  st->strings.reserve(used.size() * 3);
  for (size_t m : used) {
    auto const& src = d.mtls[m];
    sg_obj_material om{};
    std::memcpy(om.ambient, src.ambient, sizeof om.ambient);
    std::memcpy(om.diffuse, src.diffuse, sizeof om.diffuse);
    std::memcpy(om.specular, src.specular, sizeof om.specular);
    om.shininess = src.shininess;
    om.alpha = src.alpha;
    om.is_specular = src.is_specular ? 1 : 0;
    om.first_index = static_cast<uint32_t>(start[m]);
    om.index_count = static_cast<uint32_t>(start[m + 1] - start[m]);
    st->mats.push_back(om);
    st->strings.push_back(src.name);
    st->strings.push_back(src.tex_name);
    st->strings.push_back(src.tex_path);
  }
  for (size_t k = 0; k < used.size(); ++k) {
    st->mats[k].name = st->strings[k * 3].c_str();
    st->mats[k].tex_name = st->strings[k * 3 + 1].c_str();
    st->mats[k].tex_path = st->strings[k * 3 + 2].c_str();
  }
  auto h = std::make_unique<ObjMeshHolder>();
  h->pub = sg_obj_mesh{};
  h->pub.num_vertices = static_cast<uint32_t>(d.verts.size());
  h->pub.num_indices = static_cast<uint32_t>(st->indices.size());
  h->pub.num_materials = static_cast<uint32_t>(st->mats.size());
  h->pub.vertices = st->verts.data();
  h->pub.indices = st->indices.data();
  h->pub.materials = st->mats.data();
  h->store = st.release();
  *out = &h.release()->pub;
  return SG_OK;
} catch (std::bad_alloc const&) {
  return SG_OUT_OF_MEMORY;
} catch (std::exception const&) {
  return SG_FAILED;  // a path std::filesystem cannot make absolute
}

void sg_obj_release(sg_obj_mesh* mesh) {
  if (!mesh) return;
  auto* h = reinterpret_cast<ObjMeshHolder*>(mesh);
  delete h->store;
  delete h;
}

}  // extern "C"
