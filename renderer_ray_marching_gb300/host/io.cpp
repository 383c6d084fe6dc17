// io.cpp -- see io.hpp.
#include "io.hpp"

#include <zlib.h>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <fstream>
#include <iterator>
#include <sstream>
#include <stdexcept>
#include <thread>

namespace rmio {

// ------------------------------------------------------------------ PLY
namespace {

// Worker count for host-side per-point loops (PLY decoding, the radii
// archive's formatting and parsing): at 10^8 points these, not the GPU
// kernels, are what a CLI run waits for (seconds to tens of seconds on one
// thread).  Small inputs stay on the calling thread.
unsigned host_threads(size_t work) {
  if (work < ((size_t)1 << 20)) return 1;
  unsigned t = std::thread::hardware_concurrency();
  if (t == 0) t = 4;
  return std::min(t, 32u);
}

// f(slice, begin, end) over nt contiguous slices of [0, n), on nt threads;
// the first exception thrown by a slice is rethrown here.
template <class F>
void parallel_slices(size_t n, unsigned nt, F&& f) {
  if (nt <= 1) {
    f(0u, (size_t)0, n);
    return;
  }
  std::vector<std::thread> th;
  std::vector<std::exception_ptr> err(nt);
  for (unsigned c = 0; c < nt; ++c) {
    const size_t b = n * c / nt, e = n * (c + 1) / nt;
    th.emplace_back([&f, &err, c, b, e] {
      try {
        f(c, b, e);
      } catch (...) {
        err[c] = std::current_exception();
      }
    });
  }
  for (auto& t : th) t.join();
  for (auto& e : err)
    if (e) std::rethrow_exception(e);
}

inline bool is_space(char ch) { return std::isspace((unsigned char)ch) != 0; }

}  // namespace

namespace {

enum class PType { I8, U8, I16, U16, I32, U32, F32, F64 };

PType parse_ptype(const std::string& t) {
  if (t == "char" || t == "int8") return PType::I8;
  if (t == "uchar" || t == "uint8") return PType::U8;
  if (t == "short" || t == "int16") return PType::I16;
  if (t == "ushort" || t == "uint16") return PType::U16;
  if (t == "int" || t == "int32") return PType::I32;
  if (t == "uint" || t == "uint32") return PType::U32;
  if (t == "float" || t == "float32") return PType::F32;
  if (t == "double" || t == "float64") return PType::F64;
  throw std::runtime_error("PLY: unknown property type " + t);
}

int psize(PType t) {
  switch (t) {
    case PType::I8: case PType::U8: return 1;
    case PType::I16: case PType::U16: return 2;
    case PType::I32: case PType::U32: case PType::F32: return 4;
    default: return 8;
  }
}

double read_bin(const unsigned char* p, PType t, bool swap) {
  unsigned char b[8];
  int n = psize(t);
  for (int i = 0; i < n; ++i) b[i] = swap ? p[n - 1 - i] : p[i];
  switch (t) {
    case PType::I8: { int8_t v; memcpy(&v, b, 1); return v; }
    case PType::U8: { uint8_t v; memcpy(&v, b, 1); return v; }
    case PType::I16: { int16_t v; memcpy(&v, b, 2); return v; }
    case PType::U16: { uint16_t v; memcpy(&v, b, 2); return v; }
    case PType::I32: { int32_t v; memcpy(&v, b, 4); return v; }
    case PType::U32: { uint32_t v; memcpy(&v, b, 4); return v; }
    case PType::F32: { float v; memcpy(&v, b, 4); return v; }
    default: { double v; memcpy(&v, b, 8); return v; }
  }
}

struct Prop {
  std::string name;
  PType type;
  bool list = false;
  PType count_type = PType::U8;
};

struct Element {
  std::string name;
  size_t count = 0;
  std::vector<Prop> props;
};

bool host_big_endian() {
  uint16_t x = 1;
  unsigned char c;
  memcpy(&c, &x, 1);
  return c == 0;
}

uint8_t to_u8(double v, PType t) {
  if (t == PType::F32 || t == PType::F64) v = v * 255.0;
  if (v < 0) v = 0;
  if (v > 255) v = 255;
  return (uint8_t)v;
}

}  // namespace

Cloud load_ply(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("PLY: cannot open " + path);
  std::string line;
  std::getline(f, line);
  if (line.rfind("ply", 0) != 0) throw std::runtime_error("PLY: bad magic in " + path);
  std::string format;
  std::vector<Element> elems;
  while (std::getline(f, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    std::istringstream ss(line);
    std::string kw;
    ss >> kw;
    if (kw == "format") {
      ss >> format;
    } else if (kw == "element") {
      Element e;
      ss >> e.name >> e.count;
      elems.push_back(e);
    } else if (kw == "property") {
      if (elems.empty()) throw std::runtime_error("PLY: property before element");
      Prop p;
      std::string t;
      ss >> t;
      if (t == "list") {
        std::string ct, it;
        ss >> ct >> it >> p.name;
        p.list = true;
        p.count_type = parse_ptype(ct);
        p.type = parse_ptype(it);
      } else {
        p.type = parse_ptype(t);
        ss >> p.name;
      }
      elems.back().props.push_back(p);
    } else if (kw == "end_header") {
      break;
    }
  }
  bool ascii = format == "ascii";
  bool swap = (format == "binary_big_endian") != host_big_endian();
  if (!ascii && format != "binary_little_endian" && format != "binary_big_endian")
    throw std::runtime_error("PLY: unsupported format " + format);
  Cloud c;
  for (const Element& e : elems) {
    int ix = -1, iy = -1, iz = -1, ir = -1, ig = -1, ib = -1;
    bool has_list = false;
    size_t stride = 0;
    std::vector<size_t> off;
    for (size_t k = 0; k < e.props.size(); ++k) {
      const Prop& p = e.props[k];
      has_list |= p.list;
      off.push_back(stride);
      stride += psize(p.type);
      if (p.name == "x") ix = (int)k;
      if (p.name == "y") iy = (int)k;
      if (p.name == "z") iz = (int)k;
      if (p.name == "red" || p.name == "r") ir = (int)k;
      if (p.name == "green" || p.name == "g") ig = (int)k;
      if (p.name == "blue" || p.name == "b") ib = (int)k;
    }
    bool is_vertex = e.name == "vertex";
    if (is_vertex && (ix < 0 || iy < 0 || iz < 0)) throw std::runtime_error("PLY: vertex lacks x/y/z");
    if (is_vertex) {
      c.xyz.resize(e.count * 3);
      c.rgb.assign(e.count * 3, 255);
    }
    bool colour = ir >= 0 && ig >= 0 && ib >= 0;
    if (ascii) {
      for (size_t i = 0; i < e.count; ++i) {
        std::getline(f, line);
        if (!is_vertex) continue;
        std::istringstream ss(line);
        std::vector<double> vals;
        for (const Prop& p : e.props) {
          double v;
          if (p.list) {
            size_t cnt;
            ss >> cnt;
            for (size_t q = 0; q < cnt; ++q) ss >> v;
            vals.push_back(0);
          } else {
            ss >> v;
            vals.push_back(v);
          }
        }
        if (!ss) throw std::runtime_error("PLY: short ascii vertex line");
        c.xyz[3 * i + 0] = (float)vals[ix];
        c.xyz[3 * i + 1] = (float)vals[iy];
        c.xyz[3 * i + 2] = (float)vals[iz];
        if (colour) {
          c.rgb[3 * i + 0] = to_u8(vals[ir], e.props[ir].type);
          c.rgb[3 * i + 1] = to_u8(vals[ig], e.props[ig].type);
          c.rgb[3 * i + 2] = to_u8(vals[ib], e.props[ib].type);
        }
      }
    } else if (!has_list) {
      // fixed-size records: read in chunks of up to 4M records, decode each
      // chunk in parallel slices
      const size_t chunk = (size_t)1 << 22;
      std::vector<unsigned char> buf(stride * std::min<size_t>(e.count, chunk));
      size_t done = 0;
      while (done < e.count) {
        size_t m = std::min<size_t>(e.count - done, chunk);
        f.read((char*)buf.data(), (std::streamsize)(stride * m));
        if ((size_t)f.gcount() != stride * m) throw std::runtime_error("PLY: truncated " + path);
        if (is_vertex) {
          parallel_slices(m, host_threads(m), [&](unsigned, size_t jb, size_t je) {
            for (size_t j = jb; j < je; ++j) {
              const unsigned char* r = buf.data() + j * stride;
              size_t i = done + j;
              c.xyz[3 * i + 0] = (float)read_bin(r + off[ix], e.props[ix].type, swap);
              c.xyz[3 * i + 1] = (float)read_bin(r + off[iy], e.props[iy].type, swap);
              c.xyz[3 * i + 2] = (float)read_bin(r + off[iz], e.props[iz].type, swap);
              if (colour) {
                c.rgb[3 * i + 0] = to_u8(read_bin(r + off[ir], e.props[ir].type, swap), e.props[ir].type);
                c.rgb[3 * i + 1] = to_u8(read_bin(r + off[ig], e.props[ig].type, swap), e.props[ig].type);
                c.rgb[3 * i + 2] = to_u8(read_bin(r + off[ib], e.props[ib].type, swap), e.props[ib].type);
              }
            }
          });
        }
        done += m;
      }
    } else {
      if (is_vertex) throw std::runtime_error("PLY: list properties on vertices are not supported");
      // variable-size element (faces): walk it
      for (size_t i = 0; i < e.count; ++i)
        for (const Prop& p : e.props) {
          unsigned char b[8];
          if (p.list) {
            f.read((char*)b, psize(p.count_type));
            size_t cnt = (size_t)read_bin(b, p.count_type, swap);
            f.seekg((std::streamoff)(cnt * psize(p.type)), std::ios::cur);
          } else {
            f.seekg(psize(p.type), std::ios::cur);
          }
        }
    }
    if (is_vertex) break;  // nothing after the vertices is needed
  }
  return c;
}

void save_ply(const std::string& path, const Cloud& c) {
  std::ofstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("PLY: cannot write " + path);
  size_t n = c.size();
  f << "ply\nformat binary_little_endian 1.0\nelement vertex " << n
    << "\nproperty float x\nproperty float y\nproperty float z\n"
       "property uchar red\nproperty uchar green\nproperty uchar blue\nend_header\n";
  std::vector<unsigned char> rec(15 * n);
  for (size_t i = 0; i < n; ++i) {
    memcpy(&rec[15 * i], &c.xyz[3 * i], 12);
    rec[15 * i + 12] = c.rgb[3 * i];
    rec[15 * i + 13] = c.rgb[3 * i + 1];
    rec[15 * i + 14] = c.rgb[3 * i + 2];
  }
  f.write((const char*)rec.data(), (std::streamsize)rec.size());
}

// ------------------------------------------------------------------ radii archive

std::vector<float> read_radii_archive(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot open radii file " + path);
  std::string data((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  const size_t size = data.size();
  size_t pos = 0;
  auto next_token = [&](std::string* out) -> bool {
    while (pos < size && is_space(data[pos])) ++pos;
    if (pos >= size) return false;
    const size_t b = pos;
    while (pos < size && !is_space(data[pos])) ++pos;
    if (out) out->assign(data, b, pos - b);
    return true;
  };
  std::string t0, t1, ver;
  if (!next_token(&t0) || !next_token(&t1) || !next_token(&ver) || t0 != "22" ||
      t1 != "serialization::archive")
    throw std::runtime_error("radii file " + path + " is not a Boost text archive");
  const size_t body = pos;
  // token starts per slice of the body (a token starts at a non-space byte
  // that follows a space), then their prefix sums: global token numbers
  const unsigned nt = host_threads(size - body);
  std::vector<size_t> count(nt, 0), first(nt + 1, 0);
  auto starts_token = [&](size_t i) { return !is_space(data[i]) && (i == body || is_space(data[i - 1])); };
  parallel_slices(size - body, nt, [&](unsigned c, size_t b, size_t e) {
    size_t k = 0;
    for (size_t i = body + b; i < body + e; ++i) k += starts_token(i) ? 1 : 0;
    count[c] = k;
  });
  for (unsigned c = 0; c < nt; ++c) first[c + 1] = first[c] + count[c];
  const size_t ntok = first[nt];
  std::vector<std::string> head;  // up to four leading tokens, for the layout
  for (std::string t; head.size() < 4 && next_token(&t);) head.push_back(t);
  auto is_uint = [](const std::string& x) {
    return !x.empty() && std::all_of(x.begin(), x.end(), [](char ch) { return std::isdigit((unsigned char)ch); });
  };
  // candidate layouts: (leading tokens before count, tokens after count)
  const int layouts[4][2] = {{2, 1}, {2, 0}, {0, 1}, {0, 0}};
  for (auto& L : layouts) {
    const size_t lead = L[0], after = L[1];
    if (ntok < lead + 1 + after || head.size() <= lead || !is_uint(head[lead])) continue;
    const size_t n = std::stoull(head[lead]);
    if (ntok != lead + 1 + after + n) continue;
    const size_t vstart = lead + 1 + after;  // token number of the first value
    std::vector<float> out(n);
    parallel_slices(size - body, nt, [&](unsigned c, size_t b, size_t e) {
      size_t g = first[c];
      for (size_t i = body + b; i < body + e; ++i) {
        if (!starts_token(i)) continue;
        if (g >= vstart) {
          char* end = nullptr;
          out[g - vstart] = std::strtof(data.c_str() + i, &end);
          if (end == data.c_str() + i) {
            size_t j = i;
            while (j < size && !is_space(data[j])) ++j;
            throw std::runtime_error("radii file " + path + ": bad value '" + data.substr(i, j - i) + "'");
          }
        }
        ++g;
      }
    });
    return out;
  }
  throw std::runtime_error("radii file " + path + ": element count does not match its contents");
}

void write_radii_archive(const std::string& path, const std::vector<float>& radii) {
  // values are formatted in parallel slices and written in order: the bytes
  // equal those of one fprintf(" %.9e") per value
  const size_t n = radii.size();
  const unsigned nt = host_threads(n);
  std::vector<std::string> parts(nt);
  parallel_slices(n, nt, [&](unsigned c, size_t b, size_t e) {
    std::string& out = parts[c];
    out.reserve((e - b) * 17);
    char buf[48];
    for (size_t i = b; i < e; ++i) {
      const int k = snprintf(buf, sizeof(buf), " %.9e", (double)radii[i]);
      out.append(buf, (size_t)k);
    }
  });
  FILE* f = fopen(path.c_str(), "w");
  if (!f) throw std::runtime_error("cannot write radii file " + path);
  fprintf(f, "22 serialization::archive 17 0 0 %zu 0", n);
  for (const std::string& part : parts) fwrite(part.data(), 1, part.size(), f);
  fputc('\n', f);
  const bool bad = ferror(f) != 0;  // a short write (e.g. a full disk) must not pass silently
  if (fclose(f) != 0 || bad) throw std::runtime_error("cannot write radii file " + path);
}

// ------------------------------------------------------------------ JSON
const Json& Json::at(const std::string& key) const {
  auto it = obj.find(key);
  if (kind != Object || it == obj.end()) throw std::runtime_error("JSON: missing key '" + key + "'");
  return it->second;
}

namespace {
struct Parser {
  const std::string& s;
  size_t i = 0;
  explicit Parser(const std::string& t) : s(t) {}
  void ws() {
    while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
  }
  [[noreturn]] void fail(const char* what) {
    throw std::runtime_error(std::string("JSON: ") + what + " at offset " + std::to_string(i));
  }
  Json value() {
    ws();
    if (i >= s.size()) fail("unexpected end");
    char ch = s[i];
    Json j;
    if (ch == '{') {
      ++i;
      j.kind = Json::Object;
      ws();
      if (i < s.size() && s[i] == '}') { ++i; return j; }
      while (true) {
        ws();
        Json k = value();
        if (k.kind != Json::String) fail("object key is not a string");
        ws();
        if (i >= s.size() || s[i] != ':') fail("expected ':'");
        ++i;
        j.obj[k.str] = value();
        ws();
        if (i < s.size() && s[i] == ',') { ++i; continue; }
        if (i < s.size() && s[i] == '}') { ++i; break; }
        fail("expected ',' or '}'");
      }
    } else if (ch == '[') {
      ++i;
      j.kind = Json::Array;
      ws();
      if (i < s.size() && s[i] == ']') { ++i; return j; }
      while (true) {
        j.arr.push_back(value());
        ws();
        if (i < s.size() && s[i] == ',') { ++i; continue; }
        if (i < s.size() && s[i] == ']') { ++i; break; }
        fail("expected ',' or ']'");
      }
    } else if (ch == '"') {
      ++i;
      j.kind = Json::String;
      while (i < s.size() && s[i] != '"') {
        if (s[i] == '\\') {
          ++i;
          if (i >= s.size()) fail("bad escape");
          char e = s[i];
          if (e == 'n') j.str += '\n';
          else if (e == 't') j.str += '\t';
          else if (e == 'r') j.str += '\r';
          else if (e == 'b') j.str += '\b';
          else if (e == 'f') j.str += '\f';
          else if (e == 'u') {
            if (i + 4 >= s.size()) fail("bad \\u escape");
            unsigned cp = std::stoul(s.substr(i + 1, 4), nullptr, 16);
            i += 4;
            if (cp < 0x80) j.str += (char)cp;
            else if (cp < 0x800) { j.str += (char)(0xC0 | (cp >> 6)); j.str += (char)(0x80 | (cp & 0x3F)); }
            else { j.str += (char)(0xE0 | (cp >> 12)); j.str += (char)(0x80 | ((cp >> 6) & 0x3F)); j.str += (char)(0x80 | (cp & 0x3F)); }
          } else j.str += e;
          ++i;
        } else {
          j.str += s[i++];
        }
      }
      if (i >= s.size()) fail("unterminated string");
      ++i;
    } else if (s.compare(i, 4, "true") == 0) {
      i += 4; j.kind = Json::Bool; j.b = true;
    } else if (s.compare(i, 5, "false") == 0) {
      i += 5; j.kind = Json::Bool; j.b = false;
    } else if (s.compare(i, 4, "null") == 0) {
      i += 4;
    } else {
      const char* p = s.c_str() + i;
      char* end = nullptr;
      j.num = std::strtod(p, &end);
      if (end == p) fail("bad value");
      j.kind = Json::Number;
      i += (size_t)(end - p);
    }
    return j;
  }
};
}  // namespace

Json parse_json(const std::string& text) {
  Parser p(text);
  Json j = p.value();
  p.ws();
  if (p.i != text.size()) p.fail("trailing characters");
  return j;
}

Json load_json(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("cannot open " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  return parse_json(ss.str());
}

void json_mat4(const Json& j, float out[16]) {
  if (j.kind != Json::Array || j.arr.size() != 4) throw std::runtime_error("JSON: matrix must have 4 rows");
  for (int r = 0; r < 4; ++r) {
    const Json& row = j.arr[r];
    if (row.kind != Json::Array || row.arr.size() < 4) throw std::runtime_error("JSON: matrix row must have 4 values");
    // nlohmann get<std::vector<float>>: each double narrowed to float
    for (int c = 0; c < 4; ++c) out[4 * c + r] = (float)row.arr[c].num;
  }
}

// ------------------------------------------------------------------ PNG / NPY
namespace {
void put32(std::vector<unsigned char>& v, uint32_t x) {
  v.push_back((unsigned char)(x >> 24));
  v.push_back((unsigned char)(x >> 16));
  v.push_back((unsigned char)(x >> 8));
  v.push_back((unsigned char)x);
}
void chunk(std::vector<unsigned char>& out, const char* type, const unsigned char* data, size_t n) {
  put32(out, (uint32_t)n);
  size_t start = out.size();
  out.insert(out.end(), type, type + 4);
  if (n) out.insert(out.end(), data, data + n);
  uLong crc = crc32(0L, Z_NULL, 0);
  crc = crc32(crc, out.data() + start, (uInt)(4 + n));
  put32(out, (uint32_t)crc);
}
}  // namespace

namespace {
// One zlib stream (level 1) over `raw`, deflated in `slices` row-aligned
// slices on as many threads: every slice is a raw deflate stream of its own
// rows, the first ones ending on a sync flush (an empty stored block, so the
// next slice starts byte-aligned) and the last one on the final block; the
// stream's Adler-32 is combined from the slices' sums.  Each slice starts
// without the previous one's history, which costs a little compression.
std::vector<unsigned char> zlib_slices(const std::vector<unsigned char>& raw, size_t row_bytes, int slices) {
  const size_t rows = raw.size() / row_bytes;
  std::vector<std::vector<unsigned char>> part(slices);
  std::vector<uLong> sum(slices);
  std::vector<size_t> len(slices);
  std::vector<int> ok(slices, 0);
  std::vector<std::thread> workers;
  for (int t = 0; t < slices; ++t)
    workers.emplace_back([&, t] {
      const size_t b = rows * t / slices * row_bytes, e = rows * (t + 1) / slices * row_bytes;
      len[t] = e - b;
      sum[t] = adler32(adler32(0L, Z_NULL, 0), raw.data() + b, (uInt)(e - b));
      z_stream zs;
      memset(&zs, 0, sizeof(zs));
      if (deflateInit2(&zs, 1, Z_DEFLATED, -15, 8, Z_DEFAULT_STRATEGY) != Z_OK) return;
      part[t].resize(deflateBound(&zs, (uLong)(e - b)) + 64);
      zs.next_in = const_cast<unsigned char*>(raw.data() + b);
      zs.avail_in = (uInt)(e - b);
      zs.next_out = part[t].data();
      zs.avail_out = (uInt)part[t].size();
      const bool last = t == slices - 1;
      const int rc = deflate(&zs, last ? Z_FINISH : Z_SYNC_FLUSH);
      ok[t] = (last ? rc == Z_STREAM_END : rc == Z_OK) && zs.avail_in == 0;
      part[t].resize(part[t].size() - zs.avail_out);
      deflateEnd(&zs);
    });
  for (auto& w : workers) w.join();
  std::vector<unsigned char> z = {0x78, 0x01};  // deflate, 32 KB window, fastest level
  uLong a = sum[0];
  for (int t = 0; t < slices; ++t) {
    if (!ok[t]) throw std::runtime_error("PNG: deflate failed");
    z.insert(z.end(), part[t].begin(), part[t].end());
    if (t) a = adler32_combine(a, sum[t], (z_off_t)len[t]);
  }
  put32(z, (uint32_t)a);
  return z;
}
}  // namespace

void write_png(const std::string& path, int width, int height, int channels, const uint8_t* rows, int threads) {
  size_t row = (size_t)width * channels;
  std::vector<unsigned char> raw((row + 1) * height);
  for (int y = 0; y < height; ++y) {
    raw[y * (row + 1)] = 0;  // filter: none
    memcpy(&raw[y * (row + 1) + 1], rows + (size_t)y * row, row);
  }
  std::vector<unsigned char> z;
  uLongf zlen = 0;
  const int slices = (int)std::min<size_t>((size_t)std::max(threads, 1), (size_t)height);
  if (slices > 1 && raw.size() >= ((size_t)1 << 20) && raw.size() / slices < ((size_t)1 << 30)) {
    z = zlib_slices(raw, row + 1, slices);
    zlen = (uLongf)z.size();
  } else {
    zlen = compressBound((uLong)raw.size());
    z.resize(zlen);
    if (compress2(z.data(), &zlen, raw.data(), (uLong)raw.size(), 1) != Z_OK)
      throw std::runtime_error("PNG: deflate failed");
  }
  std::vector<unsigned char> out = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
  unsigned char ihdr[13];
  uint32_t w = (uint32_t)width, h = (uint32_t)height;
  unsigned char be[8] = {(unsigned char)(w >> 24), (unsigned char)(w >> 16), (unsigned char)(w >> 8), (unsigned char)w,
                         (unsigned char)(h >> 24), (unsigned char)(h >> 16), (unsigned char)(h >> 8), (unsigned char)h};
  memcpy(ihdr, be, 8);
  ihdr[8] = 8;                              // bit depth
  ihdr[9] = channels == 4 ? 6 : (channels == 3 ? 2 : 0);  // colour type
  ihdr[10] = ihdr[11] = ihdr[12] = 0;
  chunk(out, "IHDR", ihdr, 13);
  chunk(out, "IDAT", z.data(), zlen);
  chunk(out, "IEND", nullptr, 0);
  FILE* f = fopen(path.c_str(), "wb");
  if (!f || fwrite(out.data(), 1, out.size(), f) != out.size()) {
    if (f) fclose(f);
    throw std::runtime_error("cannot write " + path);
  }
  if (fclose(f) != 0) throw std::runtime_error("cannot write " + path);
}

void write_npy_f32(const std::string& path, int height, int width, const float* data) {
  std::string dict = "{'descr': '<f4', 'fortran_order': False, 'shape': (" + std::to_string(height) + ", " +
                     std::to_string(width) + "), }";
  size_t total = 10 + dict.size() + 1;
  size_t pad = (64 - total % 64) % 64;
  dict += std::string(pad, ' ') + "\n";
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot write " + path);
  const unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
  uint16_t hl = (uint16_t)dict.size();
  unsigned char hle[2] = {(unsigned char)(hl & 255), (unsigned char)(hl >> 8)};
  fwrite(magic, 1, 8, f);
  fwrite(hle, 1, 2, f);
  fwrite(dict.data(), 1, dict.size(), f);
  size_t n = (size_t)width * height;
  if (host_big_endian()) {
    for (size_t i = 0; i < n; ++i) {
      unsigned char b[4];
      memcpy(b, &data[i], 4);
      std::swap(b[0], b[3]);
      std::swap(b[1], b[2]);
      fwrite(b, 1, 4, f);
    }
  } else {
    fwrite(data, 4, n, f);
  }
  const bool bad = ferror(f) != 0;  // a short write (e.g. a full disk) must not pass silently
  if (fclose(f) != 0 || bad) throw std::runtime_error("cannot write " + path);
}

void encode_colour_rgba8(int width, int height, const float* rgbd, std::vector<uint8_t>& out) {
  out.resize((size_t)width * height * 4);
  for (int y = 0; y < height; ++y) {
    const float* src = rgbd + (size_t)(height - 1 - y) * width * 4;
    uint8_t* dst = out.data() + (size_t)y * width * 4;
    for (int x = 0; x < width; ++x) {
      for (int ch = 0; ch < 3; ++ch) dst[4 * x + ch] = (unsigned char)(src[4 * x + ch] * 255.0f);
      dst[4 * x + 3] = (unsigned char)(1.0f * 255.0f);  // alpha forced to 1 (src/utils.cu:154)
    }
  }
}

void encode_depth_u8(int width, int height, const float* rgbd, std::vector<uint8_t>& out,
                     std::vector<float>& depth_flipped) {
  size_t n = (size_t)width * height;
  out.resize(n);
  depth_flipped.resize(n);
  for (int y = 0; y < height; ++y) {
    const float* src = rgbd + (size_t)(height - 1 - y) * width * 4;
    for (int x = 0; x < width; ++x) {
      float v = src[4 * x + 3];
      depth_flipped[(size_t)y * width + x] = v;
      uint8_t px;
      if (std::abs(v - 1.0f) < 0.00001f) px = 0;
      else px = (uint8_t)std::clamp((255.0f / 100.0f) * v, 0.0f, 255.0f);
      out[(size_t)y * width + x] = px;
    }
  }
}

}  // namespace rmio
