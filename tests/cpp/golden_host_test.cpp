// This library's SimulationParameters and MaterialHandler against values made
// by the reference's own classes (tests/golden/ref_host_golden.txt, written by
// tests/golden/make_ref_golden.py from ParallelFDTD's
// src/base/SimulationParameters.cpp and MaterialHandler.cpp compiled
// unchanged).  Every value must match bit for bit.
//
// usage: golden_host_test <ref_host_golden.txt> <grid_ir_kat.txt>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "MaterialHandler.h"
#include "SimulationParameters.h"
#include "check.h"

namespace {

std::vector<float> data_f32;
std::vector<double> data_f64;
std::string grid_ir_path;

void samples_line(std::istringstream& in, bool dbl) {
  int st, it;
  unsigned fs, steps;
  in >> st >> it >> fs >> steps;
  SimulationParameters sp;
  sp.setUpdateType(SRL_FORWARD);
  sp.setNumSteps(steps);
  sp.setSpatialFs(fs);
  if (dbl)
    sp.addInputDataDouble(data_f64);
  else
    sp.addInputData(data_f32);
  if (st == SRC_TRANSPARENT) sp.readGridIr(grid_ir_path);
  sp.addSource(Source(0.f, 0.f, 0.f, (SrcType)st, (InputType)it, 0));
  for (unsigned s = 0; s < steps; ++s) {
    double want;
    in >> want;
    if (dbl) {
      CHECK_EQUAL(sp.getSourceSampleDouble(0, s), want);
    } else {
      CHECK_EQUAL(sp.getSourceSample(0, s), (float)want);
    }
  }
}

void params_line(std::istringstream& in, bool dbl) {
  std::string scheme;
  unsigned octave;
  in >> scheme >> octave;
  SimulationParameters sp;
  sp.setUpdateType(scheme == "forward" ? SRL_FORWARD : SRL);
  sp.setOctave(octave);
  double want[4];
  for (double& w : want) in >> w;
  if (dbl) {
    double* p = sp.getParameterPtrDouble();
    for (int i = 0; i < 4; ++i) CHECK_EQUAL(p[i], want[i]);
  } else {
    float* p = sp.getParameterPtr();
    for (int i = 0; i < 4; ++i) CHECK_EQUAL(p[i], (float)want[i]);
  }
}

std::vector<float> surfaces;

void table_line(std::istringstream& in, bool dbl) {
  unsigned nu, ns;
  in >> nu >> ns;
  std::vector<unsigned> idx(ns);
  for (unsigned& v : idx) in >> v;
  std::vector<double> tab(nu * 20);
  for (double& v : tab) in >> v;
  MaterialHandler mh;
  mh.addMaterials(surfaces.data(), ns, 20);
  CHECK_EQUAL(mh.getNumberOfUniqueMaterials(), nu);
  for (unsigned i = 0; i < ns; ++i) CHECK_EQUAL(mh.getMaterialIdxAt(i), idx[i]);
  if (dbl) {
    double* p = mh.getMaterialCoefficientPtrDouble();
    for (unsigned i = 0; i < nu * 20; ++i) CHECK_EQUAL(p[i], tab[i]);
  } else {
    float* p = mh.getMaterialCoefficientPtr();
    for (unsigned i = 0; i < nu * 20; ++i) CHECK_EQUAL(p[i], (float)tab[i]);
  }
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::printf("usage: %s ref_host_golden.txt grid_ir_kat.txt\n", argv[0]);
    return 2;
  }
  grid_ir_path = argv[2];
  std::ifstream f(argv[1]);
  std::string line;
  int lines = 0;
  // surfaces lines follow their table lines: read them all first
  std::vector<std::string> all;
  while (std::getline(f, line))
    if (!line.empty() && line[0] != '#') all.push_back(line);
  for (int pass = 0; pass < 2; ++pass) {
    for (const std::string& l : all) {
      std::istringstream in(l);
      std::string kind, prec;
      in >> kind >> prec;
      const bool dbl = prec == "f64";
      if (pass == 0) {
        if (kind == "data") {
          unsigned n;
          in >> n;
          std::vector<double> v(n);
          for (double& x : v) in >> x;
          if (dbl)
            data_f64 = v;
          else
            data_f32.assign(v.begin(), v.end());
        }
        continue;
      }
      if (kind == "surfaces") {
        unsigned ns;
        in >> ns;
        surfaces.assign(ns * 20, 0.f);
        for (float& v : surfaces) {
          double d;
          in >> d;
          v = (float)d;
        }
        // the table line of the same precision comes before; re-run it now
        for (const std::string& t : all) {
          std::istringstream tin(t);
          std::string tk, tp;
          tin >> tk >> tp;
          if (tk == "table" && tp == prec) {
            table_line(tin, dbl);
            ++lines;
          }
        }
      } else if (kind == "samples") {
        samples_line(in, dbl);
        ++lines;
      } else if (kind == "params") {
        params_line(in, dbl);
        ++lines;
      }
    }
  }
  std::printf("%d golden lines, %d checks, %d failures\n", lines, g_checks, g_failures);
  return g_failures == 0 && lines == 58 ? 0 : 1;
}
