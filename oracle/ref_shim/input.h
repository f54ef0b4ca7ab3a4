// Stand-in for the reference's missing <input.h> (its hot-path sources include
// it, but the file is not in the reference tree).  Test infrastructure only:
// it lets oracle/ref_build.sh compile the reference's own hot-path sources so
// that the oracle restatement can be checked against them.  Defaults follow
// the reference's InteratomicPotentialData / DiffusionData constructors
// (IoData.cpp:513-519, 626-633); everything else is set by the harness.
#ifndef A2C_REF_SHIM_INPUT_H
#define A2C_REF_SHIM_INPUT_H
struct InputFileShim {
  double eps = 1.0e-5;
  double rc = 5.35;
  double T0 = 300.0;
  double dt = 0.0;
  double a_Pd = 3.89;
  double xUb = 1.0 - 1.0e-16;
  double xLb = 1.0e-3;
  double v = 0.0;
  double Qm = 0.0;
  char foldername[256] = ".";
  char filename_base[256] = "solution";
  int restart_file_num = 0;
};
struct Input {
  InputFileShim file;
};
#endif
