// Cell and type checks of smd_pair_forces_static, in a header that both the
// CUDA file and plain host C++ compile, so the clamping can be tested on a
// CPU without running a kernel.
//
// The entry point takes raw device arrays from another framework and cannot
// check them on the host.  These functions make every index it derives from
// them stay inside its arrays, whatever the values:
//   * a coordinate gives the reference's cell int(p / cs) with the x >= n ->
//     n - 1 correction (include/algorithms/cellOpt.h:532-539) for p in
//     [0, L]; below 0 it gives cell 0 and at or beyond L cell n - 1; a
//     coordinate that is not finite gives cell 0 and sets kStaticBadPos;
//   * a type outside [0, n_types) sets kStaticBadType (the caller then skips
//     the table lookup).
// A flagged bead's force is written as NaN.
#pragma once

#ifdef __CUDACC__
#define SMD_STATIC_HD __host__ __device__ __forceinline__
#else
#define SMD_STATIC_HD inline
#endif

namespace smd_static {

constexpr int kStaticBadPos = 1;
constexpr int kStaticBadType = 2;

// Cell index along one axis, always in [0, n) for n >= 1.  The quotient is
// compared before any conversion to int, so no input reaches an out-of-range
// conversion.
SMD_STATIC_HD int cell_coord(double p, double cs, int n, int* flags) {
  const double q = p / cs;
  if (!(q == q) || q - q != 0.0) {  // NaN, or +-inf (inf - inf is NaN)
    *flags |= kStaticBadPos;
    return 0;
  }
  if (!(q >= 0.0)) return 0;
  if (q >= (double)n) return n - 1;
  const int c = (int)q;
  return c >= n ? n - 1 : c;
}

// Cell key x + y nx + z nx ny of a bead (CellOpt::build's key).
SMD_STATIC_HD int cell_key(const double p[3], const double cs[3], const int n[3], int* flags) {
  const int cx = cell_coord(p[0], cs[0], n[0], flags);
  const int cy = cell_coord(p[1], cs[1], n[1], flags);
  const int cz = cell_coord(p[2], cs[2], n[2], flags);
  return cx + cy * n[0] + cz * n[0] * n[1];
}

SMD_STATIC_HD bool type_ok(int t, int n_types) { return t >= 0 && t < n_types; }

}  // namespace smd_static
