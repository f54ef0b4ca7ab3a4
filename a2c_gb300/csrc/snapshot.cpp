// Solution snapshots in the formats of the reference's Output class
// (Output.cpp:60-90 collection header, 133-330 VTP piece + collection
// entry, 330-480 extended XYZ).  One lattice (id 0); per site: position q,
// displacement q - q0, site id, material id, tag, atomic frequency (the
// Gaussian width sigma), one species column pair (molar fraction = the
// occupancy, 1 for Pd; chemical potential = gamma, 0 for Pd).
#include <algorithm>
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

}  // extern "C"

namespace {

// The sites of the evaluator's layout: X (4 per site, Pd sites then H
// sites), occupancy and gamma on the H sites, material 0 "Pd" / 1 "H".
struct EvalSites {
  const double *X, *X0, *xH, *gamma;
  const signed char *siteid, *tag;
  long nPd;
  double pos(long i, int k) const { return X[4 * i + k]; }
  double ref(long i, int k) const { return X0 ? X0[4 * i + k] : X[4 * i + k]; }
  int sid(long i) const { return siteid ? (int)siteid[i] : (i < nPd ? 0 : 1); }
  int mid(long i) const { return i < nPd ? 0 : 1; }
  const char *name(long i) const { return i < nPd ? "Pd" : "H"; }
  int tag_of(long i) const { return tag ? (int)tag[i] : 0; }
  double sigma(long i) const { return X[4 * i + 3]; }
  double x(long i) const { return i < nPd ? 1.0 : xH[i - nPd]; }
  double g(long i) const { return (i < nPd || !gamma) ? 0.0 : gamma[i - nPd]; }
};

// The sites of a set-up lattice (a2c_lattice_sites' fields), named by
// their material (the names given, else M<id>).
struct LatticeSitesView {
  const a2c_lattice_sites *s;
  const double *gamma;
  const char *const *names;
  int nnames;
  std::vector<std::string> fallback;
  double pos(long i, int k) const { return s->q[3 * i + k]; }
  double ref(long i, int k) const { return s->q0[3 * i + k]; }
  int sid(long i) const { return s->siteid[i]; }
  int mid(long i) const { return s->matid[i]; }
  const char *name(long i) const {
    const int m = s->matid[i];
    // Output.cpp:26-33: a material without a name (none given, or "") is
    // labelled "Mat<id>"
    if (names && m >= 0 && m < nnames && names[m] && names[m][0] != '\0') return names[m];
    return (m >= 0 && m < (int)fallback.size()) ? fallback[(size_t)m].c_str() : "Mat";
  }
  int tag_of(long i) const { return s->tag[i]; }
  double sigma(long i) const { return s->sigma[i]; }
  double x(long i) const { return s->x[i]; }
  double g(long i) const { return gamma ? gamma[i] : 0.0; }
};

template <class S>
a2c_status write_frame(const a2c_snapshot_desc *d, int frame, double time, long np, const S &a) {
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
    for (long i = 0; i < np; ++i) std::fprintf(v, line.c_str(), a.pos(i, 0), a.pos(i, 1), a.pos(i, 2));
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
    int_array("SiteID", [&](long i) { return a.sid(i); });
    int_array("MaterialID", [&](long i) { return a.mid(i); });
    int_array("Tag", [&](long i) { return a.tag_of(i); });
    real_array("AtomicFrequency", [&](long i) { return a.sigma(i); });
    real_array("MolarFraction", [&](long i) { return a.x(i); });
    real_array("ChemicalPotential", [&](long i) { return a.g(i); });
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
      std::fprintf(x, head.c_str(), a.name(i));
      std::fprintf(x, r3.c_str(), a.pos(i, 0), a.pos(i, 1), a.pos(i, 2));
      std::fprintf(x, r3.c_str(), a.pos(i, 0) - a.ref(i, 0), a.pos(i, 1) - a.ref(i, 1), a.pos(i, 2) - a.ref(i, 2));
      std::fprintf(x, mid.c_str(), a.sid(i), a.sigma(i), a.tag_of(i));
      std::fprintf(x, r.c_str(), a.x(i));
      std::fprintf(x, r.c_str(), a.g(i));
      std::fprintf(x, "\n");
    }
    const bool ok = std::ferror(x) == 0;
    std::fclose(x);
    if (!ok) return A2C_ERR_INVALID;
  }
  return A2C_OK;
}

}  // namespace

extern "C" {

a2c_status a2c_snapshot_write(const a2c_snapshot_desc *d, int frame, double time, int nPd, int nH, const double *X,
                              const double *X0, const double *xH, const double *gamma, const signed char *siteid,
                              const signed char *tag) {
  if (!valid(d) || frame < 0 || nPd < 0 || nH < 0 || (nPd + nH > 0 && !X) || (nH > 0 && !xH)) return A2C_ERR_INVALID;
  const EvalSites a{X, X0, xH, gamma, siteid, tag, (long)nPd};
  return write_frame(d, frame, time, (long)nPd + nH, a);
}

a2c_status a2c_snapshot_write_lattice(const a2c_snapshot_desc *d, int frame, double time,
                                      const a2c_lattice_sites *sites, const double *gamma,
                                      const char *const *material_names, int n_materials) {
  if (!valid(d) || frame < 0 || !sites || sites->count < 0 || n_materials < 0 ||
      (sites->count > 0 && (!sites->q || !sites->q0 || !sites->siteid || !sites->matid || !sites->tag ||
                            !sites->sigma || !sites->x)))
    return A2C_ERR_INVALID;
  LatticeSitesView a{sites, gamma, material_names, n_materials, {}};
  int maxm = -1;
  for (int64_t i = 0; i < sites->count; ++i) maxm = std::max(maxm, sites->matid[i]);
  for (int m = 0; m <= maxm; ++m) a.fallback.push_back("Mat" + std::to_string(m));
  return write_frame(d, frame, time, (long)sites->count, a);
}

}  // extern "C"
