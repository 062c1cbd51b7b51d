// vh_png.cpp -- portable PNG decoder for depth images: any grayscale PNG (bit depth 1-16, with or without
// alpha, Adam7 interlaced or not) to 16-bit gray, the conversion the reference requests from WIC
// (GUID_WICPixelFormat16bppGray, include/tsdfmc/dataset_io.h:321-329).  Colour and palette images are
// rejected: a depth map is grayscale, and WIC's colour-to-gray weights are not part of this format.
//
// Written from the PNG specification (ISO/IEC 15948, W3C PNG 2nd edition) and RFC 1950/1951 (zlib, DEFLATE):
// chunk CRCs and the Adler-32 checksum are verified; Huffman codes are decoded canonically, one code length
// at a time.
#include "vh_png.h"

#include <cstdio>
#include <cstring>

namespace vh {
namespace png {
namespace {

uint32_t be32(const uint8_t* p) {
  return (static_cast<uint32_t>(p[0]) << 24) | (static_cast<uint32_t>(p[1]) << 16) | (static_cast<uint32_t>(p[2]) << 8) |
         p[3];
}

uint32_t crc32(const uint8_t* data, size_t n, uint32_t crc) {
  static uint32_t table[256];
  static bool ready = false;
  if (!ready) {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t c = i;
      for (int k = 0; k < 8; ++k) c = (c & 1U) ? (0xEDB88320U ^ (c >> 1)) : (c >> 1);
      table[i] = c;
    }
    ready = true;
  }
  crc = ~crc;
  for (size_t i = 0; i < n; ++i) crc = table[(crc ^ data[i]) & 0xffU] ^ (crc >> 8);
  return ~crc;
}

// ---- DEFLATE (RFC 1951) ----

struct BitReader {
  const uint8_t* data;
  size_t size;
  size_t pos = 0;    // byte position
  uint32_t bit = 0;  // bit position in data[pos]
  bool overrun = false;

  int get(int n) {  // n <= 16 bits, least significant first
    int v = 0;
    for (int i = 0; i < n; ++i) {
      if (pos >= size) {
        overrun = true;
        return 0;
      }
      v |= ((data[pos] >> bit) & 1) << i;
      if (++bit == 8) {
        bit = 0;
        ++pos;
      }
    }
    return v;
  }
  void align() {
    if (bit) {
      bit = 0;
      ++pos;
    }
  }
};

// canonical Huffman code: count of codes per length, symbols in code order
struct Huffman {
  uint16_t count[16];
  uint16_t symbol[320];
};

// false when the lengths over-subscribe the code space
bool build(Huffman& h, const uint8_t* lengths, int n) {
  std::memset(h.count, 0, sizeof(h.count));
  for (int i = 0; i < n; ++i) h.count[lengths[i]]++;
  h.count[0] = 0;
  int left = 1;
  for (int len = 1; len < 16; ++len) {
    left <<= 1;
    left -= h.count[len];
    if (left < 0) return false;
  }
  uint16_t offs[16];
  offs[1] = 0;
  for (int len = 1; len < 15; ++len) offs[len + 1] = offs[len] + h.count[len];
  for (int i = 0; i < n; ++i) {
    if (lengths[i]) h.symbol[offs[lengths[i]]++] = static_cast<uint16_t>(i);
  }
  return true;
}

// next symbol: the code is read one bit at a time, most significant first, and compared with the range of
// codes of each length; -1 on a bad code or input overrun
int decode(BitReader& br, const Huffman& h) {
  int code = 0, first = 0, index = 0;
  for (int len = 1; len < 16; ++len) {
    code |= br.get(1);
    if (br.overrun) return -1;
    const int count = h.count[len];
    if (code - first < count) return h.symbol[index + (code - first)];
    index += count;
    first = (first + count) << 1;
    code <<= 1;
  }
  return -1;
}

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool codes(BitReader& br, std::vector<uint8_t>& out, const Huffman& lit, const Huffman& dist, std::string& err) {
  for (;;) {
    const int sym = decode(br, lit);
    if (sym < 0) {
      err = "invalid literal/length code";
      return false;
    }
    if (sym < 256) {
      out.push_back(static_cast<uint8_t>(sym));
      continue;
    }
    if (sym == 256) return true;
    const int li = sym - 257;
    if (li >= 29) {
      err = "invalid length symbol";
      return false;
    }
    const int len = kLenBase[li] + br.get(kLenExtra[li]);
    const int ds = decode(br, dist);
    if (ds < 0 || ds >= 30) {
      err = "invalid distance code";
      return false;
    }
    const size_t d = kDistBase[ds] + static_cast<size_t>(br.get(kDistExtra[ds]));
    if (br.overrun) {
      err = "truncated DEFLATE stream";
      return false;
    }
    if (d > out.size()) {
      err = "distance beyond the start of the output";
      return false;
    }
    const size_t from = out.size() - d;
    for (int k = 0; k < len; ++k) out.push_back(out[from + k]);
  }
}

bool inflate(const uint8_t* data, size_t size, std::vector<uint8_t>& out, size_t* consumed, std::string& err) {
  BitReader br{data, size};
  int last = 0;
  do {
    last = br.get(1);
    const int type = br.get(2);
    if (br.overrun) {
      err = "truncated DEFLATE stream";
      return false;
    }
    if (type == 0) {  // stored
      br.align();
      if (br.pos + 4 > size) {
        err = "truncated stored block";
        return false;
      }
      const unsigned len = data[br.pos] | (data[br.pos + 1] << 8);
      const unsigned nlen = data[br.pos + 2] | (data[br.pos + 3] << 8);
      if ((len ^ 0xffffU) != nlen) {
        err = "stored block length check failed";
        return false;
      }
      br.pos += 4;
      if (br.pos + len > size) {
        err = "truncated stored block";
        return false;
      }
      out.insert(out.end(), data + br.pos, data + br.pos + len);
      br.pos += len;
    } else if (type == 1) {  // fixed Huffman codes
      static Huffman lit, dist;
      static bool ready = false;
      if (!ready) {
        uint8_t l[288];
        for (int i = 0; i < 144; ++i) l[i] = 8;
        for (int i = 144; i < 256; ++i) l[i] = 9;
        for (int i = 256; i < 280; ++i) l[i] = 7;
        for (int i = 280; i < 288; ++i) l[i] = 8;
        build(lit, l, 288);
        uint8_t dl[30];
        for (int i = 0; i < 30; ++i) dl[i] = 5;
        build(dist, dl, 30);
        ready = true;
      }
      if (!codes(br, out, lit, dist, err)) return false;
    } else if (type == 2) {  // dynamic Huffman codes
      const int hlit = br.get(5) + 257, hdist = br.get(5) + 1, hclen = br.get(4) + 4;
      static const uint8_t kOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
      uint8_t cl[19] = {};
      for (int i = 0; i < hclen; ++i) cl[kOrder[i]] = static_cast<uint8_t>(br.get(3));
      Huffman clh;
      if (br.overrun || hlit > 286 || hdist > 30 || !build(clh, cl, 19)) {
        err = "invalid code-length code";
        return false;
      }
      uint8_t lengths[320] = {};
      int n = 0;
      while (n < hlit + hdist) {
        const int sym = decode(br, clh);
        if (sym < 0) {
          err = "invalid code-length symbol";
          return false;
        }
        if (sym < 16) {
          lengths[n++] = static_cast<uint8_t>(sym);
          continue;
        }
        int rep = 0;
        uint8_t val = 0;
        if (sym == 16) {
          if (n == 0) {
            err = "repeat with no previous length";
            return false;
          }
          val = lengths[n - 1];
          rep = 3 + br.get(2);
        } else if (sym == 17) {
          rep = 3 + br.get(3);
        } else {
          rep = 11 + br.get(7);
        }
        if (n + rep > hlit + hdist) {
          err = "code lengths overflow";
          return false;
        }
        while (rep--) lengths[n++] = val;
      }
      if (lengths[256] == 0) {
        err = "no end-of-block code";
        return false;
      }
      Huffman lit, dist;
      if (!build(lit, lengths, hlit) || !build(dist, lengths + hlit, hdist)) {
        err = "over-subscribed Huffman code";
        return false;
      }
      if (!codes(br, out, lit, dist, err)) return false;
    } else {
      err = "invalid DEFLATE block type";
      return false;
    }
  } while (!last);
  br.align();
  *consumed = br.pos;
  return true;
}

int paeth(int a, int b, int c) {
  const int p = a + b - c;
  const int pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
  if (pa <= pb && pa <= pc) return a;
  return pb <= pc ? b : c;
}

// reverses the per-scanline filters of one (sub)image in place; rows of `stride` bytes, each preceded by its
// filter-type byte in `in`
bool unfilter(const uint8_t* in, uint8_t* out, int rows, size_t stride, int bpp, std::string& err) {
  for (int y = 0; y < rows; ++y) {
    const int type = in[y * (stride + 1)];
    const uint8_t* src = in + y * (stride + 1) + 1;
    uint8_t* row = out + y * stride;
    const uint8_t* prev = y ? out + (y - 1) * stride : nullptr;
    for (size_t i = 0; i < stride; ++i) {
      const int a = i >= static_cast<size_t>(bpp) ? row[i - bpp] : 0;
      const int b = prev ? prev[i] : 0;
      const int c = (prev && i >= static_cast<size_t>(bpp)) ? prev[i - bpp] : 0;
      int v = src[i];
      switch (type) {
        case 0: break;
        case 1: v += a; break;
        case 2: v += b; break;
        case 3: v += (a + b) >> 1; break;
        case 4: v += paeth(a, b, c); break;
        default: err = "invalid scanline filter type"; return false;
      }
      row[i] = static_cast<uint8_t>(v);
    }
  }
  return true;
}

}  // namespace

bool decode_gray16(const std::vector<uint8_t>& file, Image& img, std::string& err) {
  static const uint8_t kSig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
  if (file.size() < 8 || std::memcmp(file.data(), kSig, 8) != 0) {
    err = "not a PNG file (bad signature)";
    return false;
  }
  size_t pos = 8;
  uint32_t width = 0, height = 0;
  int depth = 0, ctype = -1, interlace = 0;
  bool have_ihdr = false, have_iend = false;
  std::vector<uint8_t> idat;
  while (pos + 12 <= file.size()) {
    const uint32_t len = be32(&file[pos]);
    if (len > file.size() - pos - 12) {
      err = "truncated chunk";
      return false;
    }
    const uint8_t* type = &file[pos + 4];
    const uint8_t* body = &file[pos + 8];
    if (crc32(type, len + 4, 0) != be32(body + len)) {
      err = "chunk CRC mismatch";
      return false;
    }
    if (!std::memcmp(type, "IHDR", 4)) {
      if (len != 13) {
        err = "bad IHDR";
        return false;
      }
      width = be32(body);
      height = be32(body + 4);
      depth = body[8];
      ctype = body[9];
      interlace = body[12];
      if (body[10] != 0 || body[11] != 0 || interlace > 1) {
        err = "unsupported compression, filter or interlace method";
        return false;
      }
      have_ihdr = true;
    } else if (!std::memcmp(type, "IDAT", 4)) {
      idat.insert(idat.end(), body, body + len);
    } else if (!std::memcmp(type, "IEND", 4)) {
      have_iend = true;
      break;
    } else if (!(type[0] & 0x20)) {  // unknown critical chunk
      if (std::memcmp(type, "PLTE", 4) != 0) {
        err = "unknown critical chunk";
        return false;
      }
    }
    pos += 12 + len;
  }
  if (!have_ihdr || !have_iend || idat.empty()) {
    err = "missing IHDR, IDAT or IEND";
    return false;
  }
  if (ctype != 0 && ctype != 4) {
    err = "depth PNG must be grayscale (colour type 0 or 4), got colour type " + std::to_string(ctype);
    return false;
  }
  const bool depth_ok = ctype == 0 ? (depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16)
                                   : (depth == 8 || depth == 16);
  if (!depth_ok || width == 0 || height == 0 || width > (1U << 16) || height > (1U << 16)) {
    err = "unsupported bit depth or size";
    return false;
  }
  // zlib wrapper (RFC 1950)
  if (idat.size() < 6 || (idat[0] & 0x0f) != 8 || ((idat[0] << 8) | idat[1]) % 31 != 0 || (idat[1] & 0x20)) {
    err = "bad zlib header";
    return false;
  }
  std::vector<uint8_t> raw;
  size_t used = 0;
  if (!inflate(idat.data() + 2, idat.size() - 2, raw, &used, err)) return false;
  if (2 + used + 4 > idat.size()) {
    err = "missing Adler-32 checksum";
    return false;
  }
  uint32_t s1 = 1, s2 = 0;
  for (uint8_t b : raw) {
    s1 = (s1 + b) % 65521U;
    s2 = (s2 + s1) % 65521U;
  }
  if (((s2 << 16) | s1) != be32(&idat[2 + used])) {
    err = "Adler-32 mismatch";
    return false;
  }
  const int channels = ctype == 4 ? 2 : 1;
  const int bits_pp = depth * channels;
  const int bpp = bits_pp >= 8 ? bits_pp / 8 : 1;
  img.width = static_cast<int>(width);
  img.height = static_cast<int>(height);
  img.pixels.assign(static_cast<size_t>(width) * height, 0);
  const uint32_t maxv = (1U << depth) - 1U;
  // Adam7 passes (x0, y0, dx, dy); a non-interlaced image is the single pass (0, 0, 1, 1)
  static const int kPass[7][4] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4},
                                  {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
  const int npass = interlace ? 7 : 1;
  size_t off = 0;
  std::vector<uint8_t> rows;
  for (int ps = 0; ps < npass; ++ps) {
    const int x0 = interlace ? kPass[ps][0] : 0, y0 = interlace ? kPass[ps][1] : 0;
    const int dx = interlace ? kPass[ps][2] : 1, dy = interlace ? kPass[ps][3] : 1;
    const int pw = static_cast<int>((width + dx - 1 - x0) / dx) * (static_cast<int>(width) > x0);
    const int ph = static_cast<int>((height + dy - 1 - y0) / dy) * (static_cast<int>(height) > y0);
    if (pw <= 0 || ph <= 0) continue;
    const size_t stride = (static_cast<size_t>(pw) * bits_pp + 7) / 8;
    const size_t need = static_cast<size_t>(ph) * (stride + 1);
    if (off + need > raw.size()) {
      err = "image data shorter than the image";
      return false;
    }
    rows.assign(static_cast<size_t>(ph) * stride, 0);
    if (!unfilter(raw.data() + off, rows.data(), ph, stride, bpp, err)) return false;
    off += need;
    for (int y = 0; y < ph; ++y) {
      const uint8_t* r = rows.data() + static_cast<size_t>(y) * stride;
      for (int x = 0; x < pw; ++x) {
        uint32_t g;
        if (depth == 16) {
          g = (static_cast<uint32_t>(r[x * 2 * channels]) << 8) | r[x * 2 * channels + 1];
        } else if (depth == 8) {
          g = r[x * channels] * 257U;
        } else {
          const size_t bitpos = static_cast<size_t>(x) * depth;
          const uint32_t v = (r[bitpos >> 3] >> (8 - depth - (bitpos & 7))) & maxv;
          g = v * 65535U / maxv;
        }
        const size_t X = static_cast<size_t>(x0 + x * dx), Y = static_cast<size_t>(y0 + y * dy);
        img.pixels[Y * width + X] = static_cast<uint16_t>(g);
      }
    }
  }
  return true;
}

bool read_file(const std::string& path, std::vector<uint8_t>& out, std::string& err) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) {
    err = "cannot open " + path;
    return false;
  }
  out.clear();
  uint8_t buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) out.insert(out.end(), buf, buf + n);
  const bool bad = std::ferror(f) != 0;
  std::fclose(f);
  if (bad) {
    err = "read error on " + path;
    return false;
  }
  return true;
}

}  // namespace png
}  // namespace vh
