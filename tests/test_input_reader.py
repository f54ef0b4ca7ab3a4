"""The input-file reader (a2c_input_read): the reference's syntax
(parser/Parser.y, parser/Lexer.l) and its defaults (IoData.cpp).  Host code
only."""
import pytest

import a2c_gb300 as A

FULL = r"""
// a2c input in the reference's syntax
/* multi-line
   comment */
under Diffusion {
  Temperature = 400.0;
  AttemptFrequency = 1.0d13;     // Fortran-style exponent
  ActivationEnergy = 0.23;
  SoluteChemicalPotential = -2.0*0.5;
}
Material[0].MaterialName = "PdH";
under Material[0] {
  under InteratomicPotential {
    File = "potentials/PdH.eam";
    Tolerance = 1.0e-5;
    CutOffDistance = (5 + 0.35);
  }
}
Time.TimeStep = 1.0e-12;
Time.MaxIts = 7/2;               // integer division, as in C
Time.MaxTime = 1/2.0;
under Output {
  Format = VTP_and_XYZ;
  Precision = High;
  Prefix = "results/";
  Solution = "run1";
  Frequency = 10;
}
under Lattice[0] {
  OAx = 3.89; OAy = 0.0; OAz = 0.0;
  OBx = 0.0;  OBy = 3.89; OBz = 0.0;
  OCx = 0.0;  OCy = 0.0;  OCz = 3.89;
  PeriodicOA = True; PeriodicOB = True; PeriodicOC = False;
  Site[0].La = 0.5;  // other objects are parsed and counted
}
Sphere[3].Radius = 80.0;
end
this text after end is never read {{{
"""


def write(tmp_path, text, name="in.txt"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_full_file(tmp_path):
    d = A.read_input(write(tmp_path, FULL))
    assert d["T"] == 400.0 and d["nu"] == 1e13 and d["Qm"] == 0.23 and d["mubd"] == -1.0
    assert d["eps"] == 1e-5 and d["rc"] == 5.35 and d["potential_file"] == "potentials/PdH.eam"
    assert d["dt"] == 1e-12 and d["max_its"] == 3 and d["max_time"] == 0.5
    assert d["output_format"] == 3 and d["output_precision"] == 2 and d["output_frequency"] == 10
    assert d["output_prefix"] == "results/" and d["output_solution"] == "run1"
    assert d["lattice_axes"] == [3.89, 0, 0, 0, 3.89, 0, 0, 0, 3.89]
    assert d["lattice_periodic"] == [1, 1, 0]
    assert d["n_assignments"] == 30 and d["n_used"] == 27


def test_defaults(tmp_path):
    d = A.read_input(write(tmp_path, "// nothing set\n"))
    assert (d["T"], d["nu"], d["Qm"], d["mubd"], d["eps"], d["rc"]) == (300.0, 0.0, 0.0, -2.0, 1e-5, 5.35)
    assert (d["dt"], d["max_time"], d["cfl"]) == (-1.0, 1e10, 0.5)
    assert d["output_format"] == 1 and d["output_precision"] == 1 and d["output_solution"] == "solution"
    assert d["lattice_axes"] == [1, 0, 0, 0, 1, 0, 0, 0, 1] and d["lattice_periodic"] == [0, 0, 0]


@pytest.mark.parametrize("text,line", [
    ("Diffusion.Temperature = 400.0\nTime.TimeStep = 1;", 2),   # missing ';'
    ("\n\nDiffusion.Temperature = 2 -5;", 3),                    # '-5' is one token, as in the lexer
    ("under Diffusion {\n Temperature = 1;\n", 3),               # unclosed group
    ("Diffusion.Temperature = 2^3;", 1),                         # '^' has no rule
])
def test_syntax_errors(tmp_path, text, line):
    with pytest.raises(A.A2CError, match=f"syntax error near line {line}"):
        A.read_input(write(tmp_path, text))


def test_type_errors_and_apply(tmp_path):
    with pytest.raises(A.A2CError, match="Output.Precision: unknown keyword"):
        A.read_input(write(tmp_path, "Output.Precision = Extreme;"))
    with pytest.raises(A.A2CError, match="Time.MaxIts: an integer"):
        A.read_input(write(tmp_path, "Time.MaxIts = 2.5;"))
    with pytest.raises(A.A2CError, match="cannot open"):
        A.read_input(str(tmp_path / "missing.txt"))
    import ctypes as C
    inp = A._native.Input()
    msg = C.create_string_buffer(128)
    assert A._native.lib().a2c_input_read(write(tmp_path, FULL).encode(), C.byref(inp), msg, 128) == 0
    p = A._native.GppParams()
    A._native.lib().a2c_gpp_default_params(C.byref(p))
    assert A._native.lib().a2c_input_apply(C.byref(inp), C.byref(p)) == 0
    assert (p.T, p.eps, p.rc) == (400.0, 1e-5, 5.35)
