// A stand-in MATLAB host for the MEX gateway (test infrastructure): builds
// the 15 input matrices of matlab/runFDTD.m from raw files, calls
// mexFunction, and writes the output matrices.
//
//   mex_host <dir> <nlhs>
//
// <dir> holds in0.bin .. in14.bin, each "<class:int32> <m:int64> <n:int64>"
// followed by m*n elements (column-major as MATLAB); outputs go to
// <dir>/out<i>.bin in the same format.  Without <dir> the gateway is called
// with no inputs (the argument check path, no GPU needed).
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "mex.h"

struct mxArray_tag {
  mxClassID cls;
  size_t m, n;
  std::vector<unsigned char> data;
};

static size_t class_size(mxClassID c) {
  switch (c) {
    case mxDOUBLE_CLASS: return 8;
    case mxSINGLE_CLASS: return 4;
    case mxUINT32_CLASS: return 4;
    default: return 1;
  }
}

mxArray* mxCreateNumericMatrix(size_t m, size_t n, mxClassID cls, mxComplexity) {
  mxArray* a = new mxArray_tag;
  a->cls = cls;
  a->m = m;
  a->n = n;
  a->data.assign(m * n * class_size(cls) + 8, 0);
  return a;
}
void mxDestroyArray(mxArray* a) { delete a; }
void* mxGetData(const mxArray* a) { return (void*)a->data.data(); }
size_t mxGetM(const mxArray* a) { return a->m; }
size_t mxGetN(const mxArray* a) { return a->n; }
size_t mxGetNumberOfElements(const mxArray* a) { return a->m * a->n; }
mxClassID mxGetClassID(const mxArray* a) { return a->cls; }

int mexPrintf(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  const int r = std::vprintf(fmt, ap);
  va_end(ap);
  return r;
}
int mexEvalString(const char*) { return 0; }
void mexErrMsgTxt(const char* msg) { throw std::runtime_error(msg); }

extern "C" bool utIsInterruptPending() { return false; }

static mxArray* read_matrix(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) throw std::runtime_error("cannot open " + path);
  int32_t cls = 0;
  int64_t m = 0, n = 0;
  if (std::fread(&cls, 4, 1, f) != 1 || std::fread(&m, 8, 1, f) != 1 || std::fread(&n, 8, 1, f) != 1) {
    std::fclose(f);
    throw std::runtime_error("bad header in " + path);
  }
  mxArray* a = mxCreateNumericMatrix((size_t)m, (size_t)n, (mxClassID)cls, mxREAL);
  const size_t bytes = (size_t)m * (size_t)n * class_size(a->cls);
  const size_t got = bytes ? std::fread(a->data.data(), 1, bytes, f) : 0;
  std::fclose(f);
  if (got != bytes) throw std::runtime_error("short read in " + path);
  return a;
}

static void write_matrix(const std::string& path, const mxArray* a) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot write " + path);
  const int32_t cls = a->cls;
  const int64_t m = (int64_t)a->m, n = (int64_t)a->n;
  std::fwrite(&cls, 4, 1, f);
  std::fwrite(&m, 8, 1, f);
  std::fwrite(&n, 8, 1, f);
  std::fwrite(a->data.data(), 1, a->m * a->n * class_size(a->cls), f);
  std::fclose(f);
}

int main(int argc, char** argv) {
  try {
    if (argc < 2) {
      mxArray* plhs[1] = {nullptr};
      mexFunction(1, plhs, 0, nullptr);
      std::printf("mex_host: returned without error\n");
      return 3;
    }
    const std::string dir = argv[1];
    const int nlhs = argc > 2 ? std::atoi(argv[2]) : 1;
    std::vector<mxArray*> in(15);
    for (int i = 0; i < 15; ++i) in[i] = read_matrix(dir + "/in" + std::to_string(i) + ".bin");
    std::vector<mxArray*> out(8, nullptr);
    mexFunction(nlhs, out.data(), 15, (const mxArray**)in.data());
    for (int i = 0; i < nlhs; ++i)
      if (out[i]) write_matrix(dir + "/out" + std::to_string(i) + ".bin", out[i]);
    for (mxArray* a : in) mxDestroyArray(a);
    for (mxArray* a : out)
      if (a) mxDestroyArray(a);
  } catch (const std::exception& e) {
    std::printf("mex_host: error: %s\n", e.what());
    return 2;
  }
  return 0;
}
