// Host driver of the per-track triangulation math (csrc/gbtri_track.cuh) for
// the CPU tests: reads tracks from a flat binary file, runs the FP64 and FP32
// instantiations of the N-view, algebraic and iterative estimators, and
// writes their outputs.  Compiled by tests/test_tri_track_host.py with nvcc
// as host code; no GPU is used.
//
// Input  (little-endian): int64 nt, int64 ncam, double P[ncam][12],
//        int64 off[nt+1], uint32 cam[no], double xy[no][2]
// Output: double nview64[nt][4], algebraic64[nt][4], iterative64[nt][3],
//         double nview32[nt][4], algebraic32[nt][4], iterative32[nt][3]
#include <cstdint>
#include <cstdio>
#include <vector>

#include "gbtri_track.cuh"

template <typename T>
struct HostViews {
  const T* P;
  const uint32_t* cam;
  const T* xy;
  int64_t b;
  __host__ __device__ void operator()(int j, const T** Pj, T* x, T* y) const {
    *Pj = P + 12 * (int64_t)cam[b + j];
    *x = xy[2 * (b + j)];
    *y = xy[2 * (b + j) + 1];
  }
};

template <typename T>
static void run(int64_t nt, const std::vector<T>& P, const std::vector<int64_t>& off, const std::vector<uint32_t>& cam,
                const std::vector<T>& xy, FILE* out) {
  std::vector<double> nv(4 * nt), al(4 * nt), it(3 * nt);
  for (int64_t t = 0; t < nt; ++t) {
    const HostViews<T> v{P.data(), cam.data(), xy.data(), off[t]};
    const int n = (int)(off[t + 1] - off[t]);
    T X[4], Y[4], Z[3];
    if (sizeof(T) == 8) gbba::nview_track<T, true>(v, n, X);  // the FP64 parity path (exact passes)
    else gbba::nview_track<T, false>(v, n, X);               // the FP32 path (one pass, series form)
    gbba::algebraic_track<T>(v, n, Y);
    gbba::iterative_track<T>(v, n, Z);
    for (int i = 0; i < 4; ++i) nv[4 * t + i] = X[i], al[4 * t + i] = Y[i];
    for (int i = 0; i < 3; ++i) it[3 * t + i] = Z[i];
  }
  fwrite(nv.data(), 8, nv.size(), out);
  fwrite(al.data(), 8, al.size(), out);
  fwrite(it.data(), 8, it.size(), out);
}

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* in = fopen(argv[1], "rb");
  FILE* out = fopen(argv[2], "wb");
  if (!in || !out) return 2;
  int64_t nt, ncam;
  if (fread(&nt, 8, 1, in) != 1 || fread(&ncam, 8, 1, in) != 1) return 2;
  std::vector<double> P(12 * ncam);
  std::vector<int64_t> off(nt + 1);
  if (fread(P.data(), 8, P.size(), in) != P.size() || fread(off.data(), 8, off.size(), in) != off.size()) return 2;
  const int64_t no = off[nt];
  std::vector<uint32_t> cam(no);
  std::vector<double> xy(2 * no);
  if (fread(cam.data(), 4, cam.size(), in) != cam.size() || fread(xy.data(), 8, xy.size(), in) != xy.size()) return 2;
  run<double>(nt, P, off, cam, xy, out);
  std::vector<float> Pf(P.begin(), P.end()), xyf(xy.begin(), xy.end());
  run<float>(nt, Pf, off, cam, xyf, out);
  fclose(out);
  return 0;
}
