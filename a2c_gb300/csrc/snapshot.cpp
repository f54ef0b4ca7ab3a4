// Solution snapshots in the formats of the reference's Output class
// (Output.cpp:60-90 collection header, 133-330 VTP piece + collection
// entry, 330-480 extended XYZ).  One lattice (id 0); per site: position q,
// displacement q - q0, site id, material id, tag, atomic frequency (the
// Gaussian width sigma), one species column pair (molar fraction = the
// occupancy, 1 for Pd; chemical potential = gamma, 0 for Pd).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "a2c_gpp.h"

namespace {

// "%s_L%d_%04d" -- the reference pads the frame number to four digits by an
// if-chain and prints it plainly from 1000 on, which is what %04d does too
std::string frame_name(const char *base, int lattice, int frame, const char *ext) {
  char buf[64];
  std::snprintf(buf, sizeof(buf), "_L%d_%04d.%s", lattice, frame, ext);
  return std::string(base) + buf;
}

std::string collection_name(const a2c_snapshot_desc *d) {
  return std::string(d->prefix) + "_L" + std::to_string(d->lattice_id) + ".pvd";
}

const char *fmt1(int precision) { return precision == 2 ? "%16.10e" : precision == 1 ? "%10.6e" : "%7.4e"; }

bool valid(const a2c_snapshot_desc *d) {
  return d && d->prefix && d->prefix[0] && (d->format >= 1 && d->format <= 3) && d->precision >= 0 &&
         d->precision <= 2 && d->lattice_id >= 0;
}

const char *basename_of(const char *path) {
  const char *s = std::strrchr(path, '/');
  return s ? s + 1 : path;
}

}  // namespace

extern "C" {

a2c_status a2c_snapshot_begin(const a2c_snapshot_desc *d) {
  if (!valid(d)) return A2C_ERR_INVALID;
  if (!(d->format & 1)) return A2C_OK;  // no VTP, no collection file
  const std::string f = collection_name(d);
  FILE *p = std::fopen(f.c_str(), "w");
  if (!p) return A2C_ERR_INVALID;
  std::fprintf(p, "<?xml version=\"1.0\"?>\n");
  std::fprintf(p, "<VTKFile type=\"Collection\" version=\"0.1\"\n");
  std::fprintf(p, "byte_order=\"LittleEndian\">\n");
  std::fprintf(p, "  <Collection>\n");
  std::fprintf(p, "  </Collection>\n");
  std::fprintf(p, "</VTKFile>\n");
  const bool ok = std::ferror(p) == 0;
  std::fclose(p);
  return ok ? A2C_OK : A2C_ERR_INVALID;
}

a2c_status a2c_snapshot_write(const a2c_snapshot_desc *d, int frame, double time, int nPd, int nH, const double *X,
                              const double *X0, const double *xH, const double *gamma, const signed char *siteid,
                              const signed char *tag) {
  if (!valid(d) || frame < 0 || nPd < 0 || nH < 0 || (nPd + nH > 0 && !X) || (nH > 0 && !xH)) return A2C_ERR_INVALID;
  const long np = (long)nPd + nH;
  auto q0 = [&](long i, int k) { return X0 ? X0[4 * i + k] : X[4 * i + k]; };
  auto sid = [&](long i) { return siteid ? (int)siteid[i] : (i < nPd ? 0 : 1); };
  auto tg = [&](long i) { return tag ? (int)tag[i] : 0; };
  auto xv = [&](long i) { return i < nPd ? 1.0 : xH[i - nPd]; };
  auto gv = [&](long i) { return (i < nPd || !gamma) ? 0.0 : gamma[i - nPd]; };
  const char *f = fmt1(d->precision);
  std::string sep = d->precision == 2 ? "  " : " ";
  if (d->format & 1) {
    const std::string full = frame_name(d->prefix, d->lattice_id, frame, "vtp");
    FILE *v = std::fopen(full.c_str(), "w");
    if (!v) return A2C_ERR_INVALID;
    std::fprintf(v, "<?xml version=\"1.0\"?>\n");
    std::fprintf(v, "<VTKFile type=\"PolyData\" version=\"0.1\"\n");
    std::fprintf(v, "byte_order=\"LittleEndian\">\n");
    std::fprintf(v, "  <PolyData>\n");
    std::fprintf(v, "    <Piece NumberOfPoints=\"%ld\">\n", np);
    std::fprintf(v, "      <Points>\n");
    std::fprintf(v, "        <DataArray type=\"Float32\" NumberOfComponents=\"3\" format=\"ascii\">\n");
    const std::string line = std::string("          ") + f + " " + f + " " + f + "\n";
    for (long i = 0; i < np; ++i) std::fprintf(v, line.c_str(), X[4 * i], X[4 * i + 1], X[4 * i + 2]);
    std::fprintf(v, "        </DataArray>\n");
    std::fprintf(v, "      </Points>\n");
    std::fprintf(v, "      <PointData Scalars=\"ScalarResults\" Vectors=\"VectorResults\">\n");
    auto int_array = [&](const char *name, auto value) {
      std::fprintf(v, "        <DataArray type=\"Int8\" NumberOfComponents=\"1\" Name=\"%s\" format=\"ascii\">\n", name);
      std::fprintf(v, "          ");
      for (long i = 0; i < np; ++i) std::fprintf(v, "%d ", value(i));
      std::fprintf(v, "\n");
      std::fprintf(v, "        </DataArray>\n");
    };
    auto real_array = [&](const char *name, auto value) {
      std::fprintf(v, "        <DataArray type=\"Float32\" NumberOfComponents=\"1\" Name=\"%s\" format=\"ascii\">\n",
                   name);
      std::fprintf(v, "          ");
      const std::string g = std::string(f) + " ";
      for (long i = 0; i < np; ++i) std::fprintf(v, g.c_str(), value(i));
      std::fprintf(v, "\n");
      std::fprintf(v, "        </DataArray>\n");
    };
    int_array("SiteID", sid);
    int_array("MaterialID", [&](long i) { return i < nPd ? 0 : 1; });
    int_array("Tag", tg);
    real_array("AtomicFrequency", [&](long i) { return X[4 * i + 3]; });
    real_array("MolarFraction", xv);
    real_array("ChemicalPotential", gv);
    std::fprintf(v, "      </PointData>\n");
    std::fprintf(v, "    </Piece>\n");
    std::fprintf(v, "  </PolyData>\n");
    std::fprintf(v, "</VTKFile>\n");
    const bool ok = std::ferror(v) == 0;
    std::fclose(v);
    if (!ok) return A2C_ERR_INVALID;
    // one more entry in the collection: overwrite its closing 27 bytes
    const std::string pf = collection_name(d);
    FILE *p = std::fopen(pf.c_str(), "r+");
    if (!p) return A2C_ERR_STATE;  // a2c_snapshot_begin first
    std::fseek(p, -27, SEEK_END);
    std::fprintf(p, "  <DataSet timestep=\"%e\" file=\"%s\"/>\n", time, basename_of(full.c_str()));
    std::fprintf(p, "  </Collection>\n");
    std::fprintf(p, "</VTKFile>\n");
    const bool okp = std::ferror(p) == 0;
    std::fclose(p);
    if (!okp) return A2C_ERR_INVALID;
  }
  if (d->format & 2) {
    const std::string full = frame_name(d->prefix, d->lattice_id, frame, "xyz");
    FILE *x = std::fopen(full.c_str(), "w");
    if (!x) return A2C_ERR_INVALID;
    std::fprintf(x, "%ld\n", np);
    std::fprintf(x, "Lattice=\"%e %e %e %e %e %e %e %e %e\" ", d->axes[0], d->axes[1], d->axes[2], d->axes[3],
                 d->axes[4], d->axes[5], d->axes[6], d->axes[7], d->axes[8]);
    std::fprintf(x, "Origin=\"%e %e %e\" ", d->origin[0], d->origin[1], d->origin[2]);
    std::fprintf(x, "pbc=\"%s %s %s\" ", d->periodic[0] ? "T" : "F", d->periodic[1] ? "T" : "F",
                 d->periodic[2] ? "T" : "F");
    std::fprintf(x, "Properties=\"species:S:1:pos:R:3:disp:R:3:type:I:1:atomic_freq:R:1:tag:I:1:");
    std::fprintf(x, "molar_frac:R:%d:", 1);
    std::fprintf(x, "chem_potent:R:%d\" ", 1);
    std::fprintf(x, "Time=%e\n", time);
    const std::string r = std::string(f) + sep;
    const std::string r3 = r + r + r;
    const std::string head = d->precision == 2 ? "%16s  " : "%16s ";
    const std::string mid = d->precision == 2 ? std::string("%4d  ") + f + "  %4d  " : std::string("%4d ") + f + " %4d ";
    for (long i = 0; i < np; ++i) {
      std::fprintf(x, head.c_str(), i < nPd ? "Pd" : "H");
      std::fprintf(x, r3.c_str(), X[4 * i], X[4 * i + 1], X[4 * i + 2]);
      std::fprintf(x, r3.c_str(), X[4 * i] - q0(i, 0), X[4 * i + 1] - q0(i, 1), X[4 * i + 2] - q0(i, 2));
      std::fprintf(x, mid.c_str(), sid(i), X[4 * i + 3], tg(i));
      std::fprintf(x, r.c_str(), xv(i));
      std::fprintf(x, r.c_str(), gv(i));
      std::fprintf(x, "\n");
    }
    const bool ok = std::ferror(x) == 0;
    std::fclose(x);
    if (!ok) return A2C_ERR_INVALID;
  }
  return A2C_OK;
}

}  // extern "C"
