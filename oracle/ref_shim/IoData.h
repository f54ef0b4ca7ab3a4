// Stand-in for the reference's <IoData.h> (test infrastructure only): the
// members its Output class reads -- output settings, material names, lattice
// axes, origin and periodicity -- under the reference's own names and types
// (IoData.h:271-274, 304-306, 425-437), without the parser that fills them.
#ifndef A2C_REF_SHIM_IODATA_H
#define A2C_REF_SHIM_IODATA_H
#include <map>
#include <string>
using std::map;  // the reference's IoData.h brings these names into scope; Output.h relies on it
using std::string;

struct OutputData {
  enum FileFormat { VTP = 0, XYZ = 1, VTP_and_XYZ = 2 } format = VTP;
  const char *prefix = "";
  const char *solution_filename_base = "solution";
  enum LowMediumHigh { LOW = 0, MEDIUM = 1, HIGH = 2 };
  int frequency = 0;
  double frequency_dt = -1.0;
  LowMediumHigh precision = HIGH;
};

struct MaterialData {
  const char *name = "";
};

struct LatticeData {
  double ax = 0, ay = 0, az = 0, bx = 0, by = 0, bz = 0, cx = 0, cy = 0, cz = 0;
  double ox = 0, oy = 0, oz = 0;
  enum Boolean { FALSE = 0, TRUE = 1 } a_periodic = FALSE, b_periodic = FALSE, c_periodic = FALSE;
};

template <class DataType>
struct ObjectMap {
  std::map<int, DataType *> dataMap;
};

struct IoData {
  OutputData output;
  ObjectMap<MaterialData> materialMap;
  ObjectMap<LatticeData> latticeMap;
};
#endif
