// Host-side data formats on either side of the path:
//   - loadParticlesFromCSV (src/main.cpp:215-275) with parseString /
//     parseStringToElements / replaceAll (src/utils.cpp:14-58,
//     include/utils.h:19-58);
//   - writePlyFile (src/main.cpp:69-114), written through RPly with
//     PLY_DEFAULT storage there: binary in the host's byte order, float32
//     x y z per vertex, a uchar-counted int list per face, 0-based indices.
// No GPU work; these run without a device.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <regex>
#include <stdexcept>
#include <string>
#include <vector>

#include "internal.h"

namespace pisurf {

// parseString: split at any separator character; an empty token is kept
// between separators, a trailing empty token is not.
static std::vector<std::string> split_titles(const std::string& input, char sep) {
  std::vector<std::string> out;
  std::string comm;
  for (char ch : input) {
    if (ch == sep) {
      out.push_back(comm);
      comm.clear();
    } else {
      comm += ch;
    }
  }
  if (!comm.empty()) out.push_back(comm);
  return out;
}

// parseStringToElements<float>: std::stof of every field.
static void split_floats(std::string input, std::vector<float>& out) {
  out.clear();
  size_t pos = input.find(',');
  while (pos != std::string::npos) {
    out.push_back(std::stof(input.substr(0, pos)));
    input = input.substr(pos + 1);
    pos = input.find(',');
  }
  if (!input.empty()) out.push_back(std::stof(input));
}

static int first_match(const std::vector<std::string>& titles, const std::regex& re) {
  for (size_t i = 0; i < titles.size(); ++i)
    if (std::regex_match(titles[i], re)) return (int)i;
  return (int)titles.size();
}

long long load_csv(const char* path, float* xyz, float* radius, long long cap, int cols[4]) {
  std::ifstream ifn(path);
  if (!ifn.good()) throw std::invalid_argument(std::string("cannot open ") + path);
  std::string line;
  std::getline(ifn, line);
  for (size_t p = line.find('"'); p != std::string::npos; p = line.find('"', p)) line.erase(p, 1);
  const std::vector<std::string> titles = split_titles(line, ',');
  const auto icase = std::regex::ECMAScript | std::regex::icase;
  const int xi = first_match(titles, std::regex("^(.*(:|_|-)( *)(x|0)(\"*)|x)$", icase));
  const int yi = first_match(titles, std::regex("^(.*(:|_|-)( *)(y|1)(\"*)|y)$", icase));
  const int zi = first_match(titles, std::regex("^(.*(:|_|-)( *)(z|2)(\"*)|z)$", icase));
  const int ri = radius ? first_match(titles, std::regex("^((.*)radius|r)$", icase)) : -1;
  cols[0] = xi, cols[1] = yi, cols[2] = zi, cols[3] = ri;
  const int nt = (int)titles.size();
  if (xi == nt || yi == nt || zi == nt) throw std::invalid_argument("failed to locate an axis column");
  if (radius && ri == nt) throw std::invalid_argument("failed to locate the radius column");
  long long n = 0;
  std::vector<float> el;
  std::getline(ifn, line);
  while (!line.empty()) {
    try {
      split_floats(line, el);
    } catch (const std::exception&) {
      throw std::invalid_argument("row " + std::to_string(n + 1) + ": a value does not parse");
    }
    const int need = std::max(std::max(xi, yi), std::max(zi, ri));
    if ((int)el.size() <= need) throw std::invalid_argument("row " + std::to_string(n + 1) + ": too few values");
    if (xyz && n < cap) {
      xyz[3 * n] = el[xi];
      xyz[3 * n + 1] = el[yi];
      xyz[3 * n + 2] = el[zi];
      if (radius) radius[n] = el[ri];
    }
    ++n;
    if (!std::getline(ifn, line)) line.clear();
  }
  return n;
}

static bool host_little_endian() {
  const uint16_t v = 1;
  unsigned char b;
  std::memcpy(&b, &v, 1);
  return b == 1;
}

void write_ply(const char* path, const float* verts, long long nv, const int32_t* tris, long long nt,
               int one_based) {
  FILE* fp = std::fopen(path, "wb");
  if (!fp) throw std::invalid_argument(std::string("cannot open ") + path);
  std::fprintf(fp,
               "ply\nformat %s 1.0\nelement vertex %lld\nproperty float32 x\nproperty float32 y\n"
               "property float32 z\nelement face %lld\nproperty list uchar int vertex_indices\nend_header\n",
               host_little_endian() ? "binary_little_endian" : "binary_big_endian", nv, nt);
  std::vector<unsigned char> buf;
  buf.reserve((size_t)(nv * 12 + nt * 13));
  auto put = [&](const void* p, size_t k) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    buf.insert(buf.end(), c, c + k);
  };
  for (long long i = 0; i < 3 * nv; ++i) put(verts + i, 4);
  const unsigned char three = 3;
  for (long long t = 0; t < nt; ++t) {
    put(&three, 1);
    for (int k = 0; k < 3; ++k) {
      const int32_t v = tris[3 * t + k] - (one_based ? 1 : 0);
      put(&v, 4);
    }
  }
  std::fwrite(buf.data(), 1, buf.size(), fp);
  const bool ok = std::ferror(fp) == 0;
  std::fclose(fp);
  if (!ok) throw std::invalid_argument(std::string("write failed: ") + path);
}

}  // namespace pisurf
