// Harness around the reference's own snapshot writer (Output.cpp:1-480,
// compiled unmodified against the single-rank shims) -- TEST INFRASTRUCTURE
// ONLY: it writes files the tests compare, byte for byte, with the
// library's VTP/PVD/XYZ writers for the same sites.
#include <IoData.h>
#include <LatticeVariables.h>
#include <Output.h>

#include <vector>

MPI_Comm a2c_comm = 0;  // Utils.cpp prints through it

extern "C" {

// One lattice of n sites written as `nframes` snapshots (times[k]) by the
// reference's Output: q, q0 (3n), sigma (n), siteid, matid, tag (n); ns
// species per site with x and gamma (n x ns, row-major); nx[i] <= ns of
// them are present at site i (the rest are padded by the writer);
// axes (9: a, b, c), origin (3), periodic (3); nmat material names ("" =
// unnamed); precision 0/1/2; format 0 VTP, 1 XYZ, 2 both.  prefix is a
// directory (with the trailing slash) or a file-name prefix.
int ref_output_write(const char *prefix, const char *base, int precision, int format, int n, const double *q,
                     const double *q0, const double *sigma, const int *siteid, const int *matid, const int *tag,
                     int ns, const int *nx, const double *x, const double *gamma, const double *axes,
                     const double *origin, const int *periodic, int nmat, const char *const *names, int nframes,
                     const double *times) {
  IoData iod;
  iod.output.prefix = prefix;
  iod.output.solution_filename_base = base;
  iod.output.precision = precision == 0 ? OutputData::LOW : precision == 1 ? OutputData::MEDIUM : OutputData::HIGH;
  iod.output.format = format == 0 ? OutputData::VTP : format == 1 ? OutputData::XYZ : OutputData::VTP_and_XYZ;
  std::vector<MaterialData> mats((size_t)nmat);
  for (int m = 0; m < nmat; ++m) {
    mats[(size_t)m].name = names[m];
    iod.materialMap.dataMap[m] = &mats[(size_t)m];
  }
  LatticeData lat;
  lat.ax = axes[0], lat.ay = axes[1], lat.az = axes[2];
  lat.bx = axes[3], lat.by = axes[4], lat.bz = axes[5];
  lat.cx = axes[6], lat.cy = axes[7], lat.cz = axes[8];
  lat.ox = origin[0], lat.oy = origin[1], lat.oz = origin[2];
  lat.a_periodic = periodic[0] ? LatticeData::TRUE : LatticeData::FALSE;
  lat.b_periodic = periodic[1] ? LatticeData::TRUE : LatticeData::FALSE;
  lat.c_periodic = periodic[2] ? LatticeData::TRUE : LatticeData::FALSE;
  iod.latticeMap.dataMap[0] = &lat;

  std::vector<LatticeVariables> LVS(1);
  LatticeVariables &LV = LVS[0];
  LV.lattice_id = 0;
  LV.size = n;
  LV.nSpecies_max = ns;
  for (int i = 0; i < n; ++i) {
    LV.q.push_back(Vec3D(q[3 * i], q[3 * i + 1], q[3 * i + 2]));
    LV.q0.push_back(Vec3D(q0[3 * i], q0[3 * i + 1], q0[3 * i + 2]));
    LV.l.push_back(Vec3D(0.0, 0.0, 0.0));
    LV.sigma.push_back(sigma[i]);
    LV.siteid.push_back(siteid[i]);
    LV.matid.push_back(matid[i]);
    LV.tag.push_back(tag[i]);
    LV.x.push_back(std::vector<double>(x + (size_t)i * ns, x + (size_t)i * ns + nx[i]));
    LV.gamma.push_back(std::vector<double>(gamma + (size_t)i * ns, gamma + (size_t)i * ns + nx[i]));
  }
  MPI_Comm comm = 0;
  Output out(comm, iod);
  for (int k = 0; k < nframes; ++k) out.OutputSolution(times[k], 1e-30, k, LVS, true);
  return 0;
}

}  // extern "C"
