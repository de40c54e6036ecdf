#include "png.h"

#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <stdexcept>

namespace kf {
namespace png {
namespace {

[[noreturn]] void fail(const char *what) { throw std::runtime_error(std::string("png: ") + what); }

// Bits of a DEFLATE stream, least significant bit of each byte first
// (RFC 1951 section 3.1.1).
class Bits {
 public:
  Bits(const uint8_t *p, size_t n) : p_(p), n_(n) {}
  unsigned bit() {
    if (left_ == 0) {
      if (pos_ >= n_) fail("compressed data ends early");
      cur_ = p_[pos_++];
      left_ = 8;
    }
    const unsigned b = cur_ & 1u;
    cur_ >>= 1;
    --left_;
    return b;
  }
  // k bits as an integer, the first bit read in the least significant place
  unsigned bits(int k) {
    unsigned v = 0;
    for (int i = 0; i < k; ++i) v |= bit() << i;
    return v;
  }
  // drops the unread bits of the current byte (start of a stored block)
  void to_byte() { left_ = 0; }
  uint8_t byte() {
    if (pos_ >= n_) fail("compressed data ends early");
    return p_[pos_++];
  }

 private:
  const uint8_t *p_;
  size_t n_, pos_ = 0;
  unsigned cur_ = 0;
  int left_ = 0;
};

// A canonical Huffman code (RFC 1951 section 3.2.2): how many codes each
// length has and the symbols sorted by (length, value).
struct Code {
  uint16_t count[16];
  uint16_t sym[320];
};

void build(Code &c, const uint8_t *len, int n) {
  std::memset(c.count, 0, sizeof c.count);
  for (int s = 0; s < n; ++s) {
    if (len[s] > 15) fail("code length above 15");
    c.count[len[s]]++;
  }
  c.count[0] = 0;
  int room = 1;  // codes still available at the current length
  for (int l = 1; l < 16; ++l) {
    room = 2 * room - c.count[l];
    if (room < 0) fail("over-subscribed Huffman code");
  }
  uint16_t next[16];
  next[1] = 0;
  for (int l = 1; l < 15; ++l) next[l + 1] = (uint16_t)(next[l] + c.count[l]);
  for (int s = 0; s < n; ++s)
    if (len[s]) c.sym[next[len[s]]++] = (uint16_t)s;
}

// One symbol: the codes of one length are consecutive integers, read most
// significant bit first, and the first code of length l+1 is twice the code
// after the last code of length l.
int decode(Bits &b, const Code &c) {
  int code = 0, first = 0, index = 0;
  for (int l = 1; l < 16; ++l) {
    code |= (int)b.bit();
    const int cnt = c.count[l];
    if (code - first < cnt) return c.sym[index + (code - first)];
    index += cnt;
    first = (first + cnt) << 1;
    code <<= 1;
  }
  fail("invalid Huffman code");
}

// Match lengths of symbols 257..285 and distances of codes 0..29 (RFC 1951
// section 3.2.5): after the first few, each group of four (lengths) or two
// (distances) shares a number of extra bits, one more than the group before.
void length_of(int sym, int &base, int &extra) {
  const int i = sym - 257;
  if (i < 8) {
    base = 3 + i;
    extra = 0;
  } else if (i < 28) {
    extra = (i - 4) / 4;
    base = ((4 + (i & 3)) << extra) + 3;
  } else {
    base = 258;
    extra = 0;
  }
}

void distance_of(int code, int &base, int &extra) {
  if (code < 4) {
    base = code + 1;
    extra = 0;
  } else {
    extra = (code - 2) / 2;
    base = ((2 + (code & 1)) << extra) + 1;
  }
}

void inflate_block(Bits &b, const Code &lit, const Code &dist, std::vector<uint8_t> &out) {
  while (true) {
    const int sym = decode(b, lit);
    if (sym < 256) {
      out.push_back((uint8_t)sym);
    } else if (sym == 256) {
      return;
    } else {
      if (sym > 285) fail("invalid length symbol");
      int lb, le;
      length_of(sym, lb, le);
      const int len = lb + (int)b.bits(le);
      const int dsym = decode(b, dist);
      if (dsym > 29) fail("invalid distance symbol");
      int db, de;
      distance_of(dsym, db, de);
      const size_t d = (size_t)db + b.bits(de);
      if (d > out.size()) fail("distance before the start of the data");
      size_t from = out.size() - d;
      for (int k = 0; k < len; ++k) out.push_back(out[from + k]);
    }
  }
}

}  // namespace

std::vector<uint8_t> inflate_zlib(const uint8_t *data, size_t size) {
  if (size < 2) fail("zlib stream too short");
  const unsigned cmf = data[0], flg = data[1];
  if ((cmf & 15) != 8 || (cmf >> 4) > 7) fail("not a deflate stream");
  if ((cmf * 256 + flg) % 31 != 0) fail("bad zlib header check");
  if (flg & 32) fail("preset dictionary not supported");
  Bits b(data + 2, size - 2);
  std::vector<uint8_t> out;
  Code fixed_lit, fixed_dist;
  bool fixed_built = false;
  bool last;
  do {
    last = b.bit() != 0;
    const unsigned type = b.bits(2);
    if (type == 0) {  // stored
      b.to_byte();
      const unsigned len = b.byte() | (unsigned)b.byte() << 8;
      const unsigned nlen = b.byte() | (unsigned)b.byte() << 8;
      if ((len ^ 0xffffu) != nlen) fail("stored block length check");
      for (unsigned k = 0; k < len; ++k) out.push_back(b.byte());
    } else if (type == 1) {  // fixed codes (RFC 1951 section 3.2.6)
      if (!fixed_built) {
        uint8_t len[288];
        for (int s = 0; s < 288; ++s) len[s] = s < 144 ? 8 : s < 256 ? 9 : s < 280 ? 7 : 8;
        build(fixed_lit, len, 288);
        uint8_t dl[30];
        for (int s = 0; s < 30; ++s) dl[s] = 5;
        build(fixed_dist, dl, 30);
        fixed_built = true;
      }
      inflate_block(b, fixed_lit, fixed_dist, out);
    } else if (type == 2) {  // dynamic codes (RFC 1951 section 3.2.7)
      const int nlit = (int)b.bits(5) + 257, ndist = (int)b.bits(5) + 1, nclen = (int)b.bits(4) + 4;
      if (nlit > 286 || ndist > 30) fail("too many codes");
      static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
      uint8_t clen[19] = {0};
      for (int k = 0; k < nclen; ++k) clen[order[k]] = (uint8_t)b.bits(3);
      Code cl;
      build(cl, clen, 19);
      uint8_t len[320] = {0};
      int k = 0;
      while (k < nlit + ndist) {
        const int sym = decode(b, cl);
        if (sym < 16) {
          len[k++] = (uint8_t)sym;
        } else {
          int rep, val = 0;
          if (sym == 16) {
            if (k == 0) fail("repeat with no previous length");
            val = len[k - 1];
            rep = 3 + (int)b.bits(2);
          } else if (sym == 17) {
            rep = 3 + (int)b.bits(3);
          } else {
            rep = 11 + (int)b.bits(7);
          }
          if (k + rep > nlit + ndist) fail("code lengths overflow");
          while (rep--) len[k++] = (uint8_t)val;
        }
      }
      if (len[256] == 0) fail("no end-of-block code");
      Code lit, dist;
      build(lit, len, nlit);
      build(dist, len + nlit, ndist);
      inflate_block(b, lit, dist, out);
    } else {
      fail("invalid block type");
    }
  } while (!last);
  return out;
}

namespace {

uint32_t be32(const uint8_t *p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }

// The Paeth predictor of PNG filter type 4.
int paeth(int a, int b, int c) {
  const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
  if (pa <= pb && pa <= pc) return a;
  return pb <= pc ? b : c;
}

}  // namespace

Image decode(const std::vector<uint8_t> &f) {
  static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
  if (f.size() < 8 || std::memcmp(f.data(), sig, 8) != 0) fail("not a PNG file");
  Image im;
  int ctype = -1, interlace = 0;
  std::vector<uint8_t> idat;
  size_t pos = 8;
  bool end = false;
  while (!end) {
    if (pos + 8 > f.size()) fail("truncated chunk");
    const uint32_t len = be32(&f[pos]);
    const char *type = (const char *)&f[pos + 4];
    if (pos + 12 + (size_t)len > f.size()) fail("truncated chunk");
    const uint8_t *d = &f[pos + 8];
    if (!std::memcmp(type, "IHDR", 4)) {
      if (len < 13) fail("short IHDR");
      im.width = (int)be32(d);
      im.height = (int)be32(d + 4);
      im.bit_depth = d[8];
      ctype = d[9];
      interlace = d[12];
      if (d[10] != 0 || d[11] != 0) fail("unknown compression or filter method");
    } else if (!std::memcmp(type, "IDAT", 4)) {
      idat.insert(idat.end(), d, d + len);
    } else if (!std::memcmp(type, "IEND", 4)) {
      end = true;
    }
    pos += 12 + (size_t)len;
  }
  switch (ctype) {
    case 0: im.channels = 1; break;
    case 2: im.channels = 3; break;
    case 4: im.channels = 2; break;
    case 6: im.channels = 4; break;
    default: fail("unsupported colour type (palette or missing IHDR)");
  }
  if (im.bit_depth != 8 && im.bit_depth != 16) fail("unsupported bit depth");
  if (interlace != 0) fail("interlaced images are not supported");
  if (im.width <= 0 || im.height <= 0 || im.width > (1 << 24) || im.height > (1 << 24)) fail("bad image size");
  const std::vector<uint8_t> raw = inflate_zlib(idat.data(), idat.size());
  const int bps = im.bit_depth / 8;                  // bytes per sample
  const size_t bpp = (size_t)im.channels * bps;     // bytes per pixel
  const size_t stride = (size_t)im.width * bpp;
  if (raw.size() < (size_t)im.height * (stride + 1)) fail("image data too short");
  std::vector<uint8_t> prev(stride, 0), cur(stride);
  im.samples.resize((size_t)im.width * im.height * im.channels);
  for (int y = 0; y < im.height; ++y) {
    const uint8_t *row = &raw[(size_t)y * (stride + 1)];
    const int filter = row[0];
    for (size_t x = 0; x < stride; ++x) {
      const int v = row[1 + x];
      const int a = x >= bpp ? cur[x - bpp] : 0, b = prev[x], c = x >= bpp ? prev[x - bpp] : 0;
      int r;
      switch (filter) {
        case 0: r = v; break;
        case 1: r = v + a; break;
        case 2: r = v + b; break;
        case 3: r = v + ((a + b) >> 1); break;
        case 4: r = v + paeth(a, b, c); break;
        default: fail("unknown scanline filter");
      }
      cur[x] = (uint8_t)r;
    }
    uint16_t *out = &im.samples[(size_t)y * im.width * im.channels];
    if (bps == 1)
      for (size_t s = 0; s < stride; ++s) out[s] = cur[s];
    else
      for (size_t s = 0; s < stride / 2; ++s) out[s] = (uint16_t)(cur[2 * s] << 8 | cur[2 * s + 1]);
    prev.swap(cur);
  }
  return im;
}

Image read(const std::string &path) {
  std::ifstream in(path, std::ios::binary);
  if (!in) throw std::runtime_error("png: cannot open " + path);
  std::vector<uint8_t> f((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
  return decode(f);
}

}  // namespace png
}  // namespace kf
