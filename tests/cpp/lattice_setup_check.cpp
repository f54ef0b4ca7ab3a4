// Builds the lattices of an input file through the reference-named host
// API (a2c_host.hpp SetupLatticeVariables) and prints, as one JSON line,
// each lattice's site count and a checksum of its positions, tags, widths
// and occupancies.  Host code only: no GPU is used.
#include <cstdio>
#include <cstdlib>

#include "a2c_host.hpp"

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  std::vector<a2c_gb300::LatticeSites> LVS;
  char msg[256] = {0};
  const int st = a2c_gb300::SetupLatticeVariables(argv[1], std::atoi(argv[2]), LVS, msg, sizeof(msg));
  std::printf("{\"status\": %d, \"message\": \"%s\", \"lattices\": [", st, msg);
  for (size_t k = 0; k < LVS.size(); ++k) {
    double sq = 0.0, st2 = 0.0, ss = 0.0, sx = 0.0;
    for (double v : LVS[k].q) sq += v;
    for (int v : LVS[k].tag) st2 += v;
    for (double v : LVS[k].sigma) ss += v;
    for (double v : LVS[k].x) sx += v;
    std::printf("%s{\"n\": %lld, \"sum_q\": %.17g, \"sum_tag\": %.17g, \"sum_sigma\": %.17g, \"sum_x\": %.17g}",
                k ? ", " : "", (long long)LVS[k].size(), sq, st2, ss, sx);
  }
  std::printf("]}\n");
  return st == 0 ? 0 : 1;
}
