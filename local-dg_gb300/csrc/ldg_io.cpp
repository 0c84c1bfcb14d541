// X-Y-Z-V CSV snapshots in the reference's format (io.cpp:8-72), written by
// host threads: the state is read back once, the lines of consecutive
// element blocks are formatted in parallel and written in element order.
#include "ldg_io.hpp"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace ldg {

namespace {

// One double as "operator<<(ostream&, double)" prints it with the default
// flags and precision 6: the %g conversion with 6 significant digits.
inline int put_double(char* out, double v) { return std::snprintf(out, 32, "%.6g", v); }

struct Block {
  long e0 = 0, e1 = 0;
  std::string text;
};

void format_block(Block* b, const Geometry& g, const double* u) {
  const int N = g.N, n = N * N * N;
  std::string& t = b->text;
  t.clear();
  t.reserve((size_t)(b->e1 - b->e0) * n * 112);
  char line[8 * 32 + 16];
  for (long k = b->e0; k < b->e1; ++k) {
    const int ix = (int)(k % g.nx), iy = (int)((k / g.nx) % g.ny), iz = (int)(k / ((long)g.nx * g.ny));
    // element vertices (mesh.cpp:128-146) and node placement (mesh.cpp:396-407)
    const double x0 = ix * (g.hi[0] - g.lo[0]) / g.nx + g.lo[0], x1 = (ix + 1) * (g.hi[0] - g.lo[0]) / g.nx + g.lo[0];
    const double y0 = iy * (g.hi[1] - g.lo[1]) / g.ny + g.lo[1], y1 = (iy + 1) * (g.hi[1] - g.lo[1]) / g.ny + g.lo[1];
    const double z0 = iz * (g.hi[2] - g.lo[2]) / g.nz + g.lo[2], z1 = (iz + 1) * (g.hi[2] - g.lo[2]) / g.nz + g.lo[2];
    for (int i = 0; i < n; ++i) {
      const int c0 = i % N, c1 = (i / N) % N, c2 = i / (N * N);
      const double xyz[3] = {x0 + .5 * (g.xi[c0] + 1.0) * (x1 - x0), y0 + .5 * (g.xi[c1] + 1.0) * (y1 - y0),
                             z0 + .5 * (g.xi[c2] + 1.0) * (z1 - z0)};
      int len = 0;
      for (int l = 0; l < 3; ++l) {
        len += put_double(line + len, xyz[l]);
        line[len++] = ',';
        line[len++] = ' ';
      }
      for (int v = 0; v < 5; ++v) {
        len += put_double(line + len, u[((size_t)k * 5 + v) * n + i]);
        if (v < 4) {
          line[len++] = ',';
          line[len++] = ' ';
        }
      }
      line[len++] = '\n';
      t.append(line, (size_t)len);
    }
  }
}

}  // namespace

int write_xyzv_file(const std::string& path, const Geometry& g, const double* u) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) {
    set_last_error("cannot open " + path + " for writing");
    return LDG_ERR_IO;
  }
  // header (io.cpp:17-21)
  static const char kHeader[] = "X, Y, Z, u0, u1, u2, u3, u4\n";
  bool ok = std::fwrite(kHeader, 1, sizeof(kHeader) - 1, f) == sizeof(kHeader) - 1;
  const long nE = (long)g.nx * g.ny * g.nz;
  const int threads = (int)std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  const long per = std::max(1L, 65536L / (g.N * g.N * g.N));  // elements per block (~64k lines)
  std::vector<Block> blocks(threads);
  for (long e = 0; e < nE && ok;) {
    int used = 0;
    for (; used < threads && e < nE; ++used) {
      blocks[used].e0 = e;
      blocks[used].e1 = std::min(nE, e + per);
      e = blocks[used].e1;
    }
    std::vector<std::thread> pool;
    for (int t = 1; t < used; ++t) pool.emplace_back(format_block, &blocks[t], std::cref(g), u);
    format_block(&blocks[0], g, u);
    for (auto& th : pool) th.join();
    for (int t = 0; t < used && ok; ++t)
      ok = std::fwrite(blocks[t].text.data(), 1, blocks[t].text.size(), f) == blocks[t].text.size();
  }
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) {
    set_last_error("short write to " + path);
    return LDG_ERR_IO;
  }
  return LDG_OK;
}

}  // namespace ldg

extern "C" int ldg_write_xyzv(ldg_solver* s, const char* filename, int timeseries) {
  if (!s || !filename || !*filename) {
    ldg::set_last_error("ldg_write_xyzv: null solver or empty file name");
    return LDG_ERR_INVALID;
  }
  ldg::Geometry g;
  int st = ldg::solver_geometry(s, &g);
  if (st) return st;
  ldg_info info;
  if ((st = ldg_get_info(s, &info))) return st;
  std::vector<double> u((size_t)info.nelements * 5 * info.dofs);
  if ((st = ldg_get_state(s, u.data(), LDG_HOST))) return st;
  std::string path = filename;
  if (timeseries >= 0) path += "." + std::to_string(timeseries);  // io.cpp:30-35
  return ldg::write_xyzv_file(path, g, u.data());
}
