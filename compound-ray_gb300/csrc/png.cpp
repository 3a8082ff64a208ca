// PNG decoding for glTF base-colour textures.
//
// A self-contained reader of the PNG format (ISO/IEC 15948) with its own
// DEFLATE decompressor (RFC 1950/1951): stored, fixed-Huffman and
// dynamic-Huffman blocks, canonical Huffman codes decoded length by length.
// Supports plain and Adam7-interlaced images of every colour type at 8 bits
// per sample, 16 bits per sample (reduced to the high byte), and palette /
// grey images of 1, 2 and 4 bits; the result is always RGBA8 with the
// channel expansion of a forced 4-component load (grey g -> (g, g, g, 255),
// palette entries with their tRNS alpha).
#include "png.hpp"

#include <cstring>
#include <stdexcept>

namespace cr {
namespace {

struct Bits {
  const uint8_t* p;
  size_t n, pos = 0;
  uint32_t buf = 0;
  int cnt = 0;
  int bit() {
    if (cnt == 0) {
      if (pos >= n) throw std::runtime_error("deflate stream ends early");
      buf = p[pos++];
      cnt = 8;
    }
    const int b = static_cast<int>(buf & 1u);
    buf >>= 1;
    --cnt;
    return b;
  }
  uint32_t bits(int k) {
    uint32_t v = 0;
    for (int i = 0; i < k; ++i) v |= static_cast<uint32_t>(bit()) << i;
    return v;
  }
  void alignByte() { cnt = 0; }
};

// Canonical Huffman code: number of codes of each length and the symbols in
// code order.
struct Huffman {
  uint16_t count[16] = {0};
  uint16_t symbol[320] = {0};
  void build(const uint8_t* lengths, int n) {
    std::memset(count, 0, sizeof(count));
    for (int i = 0; i < n; ++i) ++count[lengths[i]];
    count[0] = 0;
    uint16_t offs[16];
    offs[1] = 0;
    for (int l = 1; l < 15; ++l) offs[l + 1] = static_cast<uint16_t>(offs[l] + count[l]);
    for (int i = 0; i < n; ++i)
      if (lengths[i]) symbol[offs[lengths[i]]++] = static_cast<uint16_t>(i);
  }
  int decode(Bits& b) const {
    int code = 0, first = 0, index = 0;
    for (int len = 1; len < 16; ++len) {
      code |= b.bit();
      const int c = count[len];
      if (code - c < first) return symbol[index + (code - first)];
      index += c;
      first += c;
      first <<= 1;
      code <<= 1;
    }
    throw std::runtime_error("bad Huffman code");
  }
};

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

void inflateBlock(Bits& b, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out) {
  for (;;) {
    int sym = lit.decode(b);
    if (sym < 256) {
      out.push_back(static_cast<uint8_t>(sym));
    } else if (sym == 256) {
      return;
    } else {
      sym -= 257;
      if (sym >= 29) throw std::runtime_error("bad length code");
      const size_t len = kLenBase[sym] + b.bits(kLenExtra[sym]);
      const int ds = dist.decode(b);
      if (ds >= 30) throw std::runtime_error("bad distance code");
      const size_t d = kDistBase[ds] + b.bits(kDistExtra[ds]);
      if (d > out.size()) throw std::runtime_error("distance too far back");
      const size_t from = out.size() - d;
      for (size_t i = 0; i < len; ++i) out.push_back(out[from + i]);
    }
  }
}

std::vector<uint8_t> zlibInflate(const uint8_t* p, size_t n) {
  if (n < 2) throw std::runtime_error("short zlib stream");
  if ((p[0] & 0x0F) != 8 || ((static_cast<unsigned>(p[0]) << 8) | p[1]) % 31 != 0)
    throw std::runtime_error("bad zlib header");
  if (p[1] & 0x20) throw std::runtime_error("zlib preset dictionary not supported");
  Bits b{p + 2, n - 2};
  std::vector<uint8_t> out;
  int last = 0;
  while (!last) {
    last = b.bit();
    const uint32_t type = b.bits(2);
    if (type == 0) {
      b.alignByte();
      if (b.pos + 4 > b.n) throw std::runtime_error("short stored block");
      const uint32_t len = b.p[b.pos] | (b.p[b.pos + 1] << 8);
      const uint32_t nlen = b.p[b.pos + 2] | (b.p[b.pos + 3] << 8);
      b.pos += 4;
      if ((len ^ 0xFFFFu) != nlen) throw std::runtime_error("bad stored block length");
      if (b.pos + len > b.n) throw std::runtime_error("short stored block");
      out.insert(out.end(), b.p + b.pos, b.p + b.pos + len);
      b.pos += len;
    } else if (type == 1) {
      uint8_t l[288], d[30];
      for (int i = 0; i < 144; ++i) l[i] = 8;
      for (int i = 144; i < 256; ++i) l[i] = 9;
      for (int i = 256; i < 280; ++i) l[i] = 7;
      for (int i = 280; i < 288; ++i) l[i] = 8;
      for (int i = 0; i < 30; ++i) d[i] = 5;
      Huffman lit, dist;
      lit.build(l, 288);
      dist.build(d, 30);
      inflateBlock(b, lit, dist, out);
    } else if (type == 2) {
      const int hlit = static_cast<int>(b.bits(5)) + 257, hdist = static_cast<int>(b.bits(5)) + 1,
                hclen = static_cast<int>(b.bits(4)) + 4;
      static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
      uint8_t cl[19] = {0};
      for (int i = 0; i < hclen; ++i) cl[order[i]] = static_cast<uint8_t>(b.bits(3));
      Huffman clh;
      clh.build(cl, 19);
      uint8_t lens[320] = {0};
      int i = 0;
      while (i < hlit + hdist) {
        const int sym = clh.decode(b);
        if (sym < 16) {
          lens[i++] = static_cast<uint8_t>(sym);
        } else {
          int rep = 0;
          uint8_t val = 0;
          if (sym == 16) {
            if (i == 0) throw std::runtime_error("repeat with no previous length");
            val = lens[i - 1];
            rep = 3 + static_cast<int>(b.bits(2));
          } else if (sym == 17) {
            rep = 3 + static_cast<int>(b.bits(3));
          } else {
            rep = 11 + static_cast<int>(b.bits(7));
          }
          if (i + rep > hlit + hdist) throw std::runtime_error("too many code lengths");
          while (rep--) lens[i++] = val;
        }
      }
      Huffman lit, dist;
      lit.build(lens, hlit);
      dist.build(lens + hlit, hdist);
      inflateBlock(b, lit, dist, out);
    } else {
      throw std::runtime_error("bad deflate block type");
    }
  }
  return out;
}

uint32_t be32(const uint8_t* p) {
  return (static_cast<uint32_t>(p[0]) << 24) | (static_cast<uint32_t>(p[1]) << 16) | (static_cast<uint32_t>(p[2]) << 8) | p[3];
}

int paeth(int a, int b, int c) {
  const int p = a + b - c;
  const int pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
  if (pa <= pb && pa <= pc) return a;
  if (pb <= pc) return b;
  return c;
}

}  // namespace

bool isPng(const uint8_t* data, size_t size) {
  static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
  return size >= 8 && std::memcmp(data, sig, 8) == 0;
}

Image decodePng(const uint8_t* data, size_t size) {
  if (!isPng(data, size)) throw std::runtime_error("not a PNG image");
  size_t pos = 8;
  uint32_t w = 0, h = 0;
  int depth = 0, ctype = -1, interlace = 0;
  std::vector<uint8_t> idat, palette, trns;
  while (pos + 8 <= size) {
    const uint32_t len = be32(data + pos);
    const uint8_t* type = data + pos + 4;
    if (pos + 12 + static_cast<size_t>(len) > size) throw std::runtime_error("truncated PNG chunk");
    const uint8_t* body = data + pos + 8;
    if (std::memcmp(type, "IHDR", 4) == 0) {
      if (len < 13) throw std::runtime_error("bad IHDR");
      w = be32(body);
      h = be32(body + 4);
      depth = body[8];
      ctype = body[9];
      interlace = body[12];
    } else if (std::memcmp(type, "PLTE", 4) == 0) {
      palette.assign(body, body + len);
    } else if (std::memcmp(type, "tRNS", 4) == 0) {
      trns.assign(body, body + len);
    } else if (std::memcmp(type, "IDAT", 4) == 0) {
      idat.insert(idat.end(), body, body + len);
    } else if (std::memcmp(type, "IEND", 4) == 0) {
      break;
    }
    pos += 12 + static_cast<size_t>(len);
  }
  if (w == 0 || h == 0 || w > 65536 || h > 65536) throw std::runtime_error("bad PNG size");
  if (interlace != 0 && interlace != 1) throw std::runtime_error("bad PNG interlace method");
  int channels;
  switch (ctype) {
    case 0: channels = 1; break;
    case 2: channels = 3; break;
    case 3: channels = 1; break;
    case 4: channels = 2; break;
    case 6: channels = 4; break;
    default: throw std::runtime_error("bad PNG colour type");
  }
  const bool okDepth = depth == 8 || depth == 16 || ((ctype == 0 || ctype == 3) && (depth == 1 || depth == 2 || depth == 4));
  if (!okDepth) throw std::runtime_error("unsupported PNG bit depth");
  const std::vector<uint8_t> raw = zlibInflate(idat.data(), idat.size());
  const size_t bitsPerPixel = static_cast<size_t>(channels) * depth;
  const size_t bpp = std::max<size_t>(1, bitsPerPixel / 8);
  Image img;
  img.width = static_cast<int>(w);
  img.height = static_cast<int>(h);
  img.bits = depth == 16 ? 16 : 8;
  img.rgba.resize(static_cast<size_t>(w) * h * 4);
  size_t at = 0;  // read position in the inflated stream

  // One (sub-)image of pw x ph pixels whose pixel (x, y) lands at
  // (x0 + x*dx, y0 + y*dy); each has its own filtered scanlines.
  auto pass = [&](uint32_t x0, uint32_t y0, uint32_t dx, uint32_t dy) {
    if (x0 >= w || y0 >= h) return;
    const uint32_t pw = (w - x0 + dx - 1) / dx, ph = (h - y0 + dy - 1) / dy;
    const size_t stride = (static_cast<size_t>(pw) * bitsPerPixel + 7) / 8;
    if (raw.size() - at < (stride + 1) * ph) throw std::runtime_error("PNG image data too short");
    std::vector<uint8_t> cur(stride), prev(stride, 0);
    for (uint32_t y = 0; y < ph; ++y) {
      const uint8_t* line = raw.data() + at;
      at += stride + 1;
      const int filter = line[0];
      for (size_t i = 0; i < stride; ++i) {
        const int x = line[1 + i];
        const int a = i >= bpp ? cur[i - bpp] : 0;
        const int b = prev[i];
        const int c = i >= bpp ? prev[i - bpp] : 0;
        int v;
        switch (filter) {
          case 0: v = x; break;
          case 1: v = x + a; break;
          case 2: v = x + b; break;
          case 3: v = x + ((a + b) >> 1); break;
          case 4: v = x + paeth(a, b, c); break;
          default: throw std::runtime_error("bad PNG filter");
        }
        cur[i] = static_cast<uint8_t>(v & 0xFF);
      }
      for (uint32_t x = 0; x < pw; ++x) {
        uint8_t px[4] = {0, 0, 0, 255};
        auto sample = [&](int c) -> int {
          if (depth == 8) return cur[static_cast<size_t>(x) * channels + c];
          if (depth == 16) return cur[(static_cast<size_t>(x) * channels + c) * 2];  // high byte
          const size_t bit = static_cast<size_t>(x) * depth;
          const int v = (cur[bit / 8] >> (8 - depth - (bit % 8))) & ((1 << depth) - 1);
          return ctype == 3 ? v : (v * 255) / ((1 << depth) - 1);
        };
        if (ctype == 3) {
          const int idx = sample(0);
          if (static_cast<size_t>(idx) * 3 + 2 >= palette.size())
            throw std::runtime_error("PNG palette index out of range");
          px[0] = palette[3 * idx];
          px[1] = palette[3 * idx + 1];
          px[2] = palette[3 * idx + 2];
          if (static_cast<size_t>(idx) < trns.size()) px[3] = trns[idx];
        } else if (ctype == 0 || ctype == 4) {
          px[0] = px[1] = px[2] = static_cast<uint8_t>(sample(0));
          if (ctype == 4) px[3] = static_cast<uint8_t>(sample(1));
        } else {
          px[0] = static_cast<uint8_t>(sample(0));
          px[1] = static_cast<uint8_t>(sample(1));
          px[2] = static_cast<uint8_t>(sample(2));
          if (ctype == 6) px[3] = static_cast<uint8_t>(sample(3));
        }
        const size_t X = x0 + static_cast<size_t>(x) * dx, Y = y0 + static_cast<size_t>(y) * dy;
        std::memcpy(&img.rgba[(Y * w + X) * 4], px, 4);
      }
      prev.swap(cur);
    }
  };
  if (interlace == 0) {
    pass(0, 0, 1, 1);
  } else {
    // Adam7: the seven passes' origins and spacings.
    static const uint32_t kAdam7[7][4] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4},
                                          {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
    for (const auto& p : kAdam7) pass(p[0], p[1], p[2], p[3]);
  }
  return img;
}

}  // namespace cr
