// Host-side check of the sweep tiles' bulk-copy boxes (test infrastructure).
// For every tile of a set of grid sizes whose box the kernel would copy
// (TmaBox::inside / StripBox::inside): the box's x origin is a multiple of 16
// bytes, the box lies inside the grid, and every element the tile reads from
// the box lies inside it.  Prints "ok <boxes checked>" or the first failure.
#include <cstdio>

#include "../../astrea_gb300/csrc/sweep.cuh"

using namespace astrea;

static long long g_checked = 0;

#define REQUIRE(c)                                                                                      \
  do {                                                                                                  \
    if (!(c)) {                                                                                         \
      std::printf("FAIL %s line %d: T=%d SCH=%d AX=%d TS=%d TT=%d n0=%d n1=%d s0=%d t0=%d\n", #c, __LINE__, \
                  (int)sizeof(T), SCH, AX, TS, TT, n0, n1, s0, t0);                                     \
      return false;                                                                                     \
    }                                                                                                   \
  } while (0)

template <typename T, int SCH, int AX, int TS, int TT> bool check_grid(int n0, int n1) {
  using G = Geom<SCH, 2, TS, TT>;
  using B = TmaBox<T, SCH, 2, AX, TS, TT, 1>;
  using SB = StripBox<T, AX, TS, TT>;
  const int Ns = AX == 0 ? n0 : n1, Nt = AX == 0 ? n1 : n0;
  for (int s0 = 0; s0 < Ns; s0 += TS)
    for (int t0 = 0; t0 < Nt; t0 += TT) {
      if (B::inside(s0, t0, n0, n1)) {
        ++g_checked;
        const int x = B::x0(s0, t0), y = AX == 1 ? t0 - G::WT : s0 + G::W_BEG, xo = B::xoff(t0);
        REQUIRE((x * (int)sizeof(T)) % 16 == 0);
        REQUIRE(x >= 0 && y >= 0 && x + B::BW <= n1 && y + B::BH <= n0);
        // the staged level: WW columns along the sweep, WH rows across, read at offset xo
        if (AX == 1) REQUIRE(xo >= 0 && xo + G::WW <= B::BW && G::WH <= B::BH);
        else REQUIRE(xo >= 0 && xo + G::WH <= B::BW && G::WW <= B::BH);
        // and those are the tile's virtual cells [s0+W_BEG, s0+TS+W_END) x [t0-WT, t0+TT+WT)
        if (AX == 1) REQUIRE(x + xo == s0 + G::W_BEG);
        else REQUIRE(x + xo == t0 - G::WT);
        // axis 0 reads the level in place (WLayout<true>): element (row r, column c) of the
        // level is grid cell (s0 + W_BEG + c, t0 - WT + r) of the box
        if (AX == 0) {
          using WL = WLayout<true, G, B>;
          for (int c = 0; c < G::WW; ++c)
            for (int r = 0; r < G::WH; ++r) {
              const int e = r * WL::PR + c * WL::PC + xo;
              REQUIRE(e >= 0 && e < B::BW * B::BH);
              REQUIRE(x + e % B::BW == t0 - G::WT + r && y + e / B::BW == s0 + G::W_BEG + c);
            }
        }
      }
      if (SCH == PPM && SB::inside(s0, t0, n0, n1)) {
        ++g_checked;
        const int x = SB::x0(s0, t0), y = SB::y0(s0, t0);
        REQUIRE((x * (int)sizeof(T)) % 16 == 0);
        REQUIRE(x >= 0 && y >= 0 && x + SB::BW <= n1 && y + SB::BH <= n0);
        for (int c = s0 - 1; c <= s0 + TS; ++c)
          for (int r = t0; r < t0 + TT; ++r) {
            const int e = SB::at(0, c, r, s0, t0);
            REQUIRE(e >= 0 && e < SB::BW * SB::BH);
            // the element is the grid cell (c, r): axis 0 = sweep for AX=0, rows for AX=1
            const int gx = x + e % SB::BW, gy = y + e / SB::BW;
            if (AX == 1) REQUIRE(gx == c && gy == r);
            else REQUIRE(gx == r && gy == c);
          }
      }
    }
  return true;
}

template <typename T, int SCH, int AX, int TS, int TT> bool check_all() {
  const int sizes[][2] = {{2048, 2048}, {1024, 1024}, {512, 512}, {100, 136}, {96, 64}, {64, 200}, {130, 130},
                          {33, 48}, {40, 56}, {256, 40}, {48, 1000}, {17, 20}};
  for (auto& sz : sizes)
    if (!check_grid<T, SCH, AX, TS, TT>(sz[0], sz[1])) return false;
  return true;
}

// the axis-0 box of NV planes, aligned up to 128 bytes, fits the w level's region of the WSIN tiles
template <typename T, int SCH, int TS, int TT, int NV> constexpr bool box_fits_w() {
  return SCH < PPM || (size_t)Smem<SCH, 2, TS, TT, NV, true>::n_w * sizeof(T) >=
                          (size_t)TmaBox<T, SCH, 2, 0, TS, TT, NV>::BYTES + 128;
}
static_assert(box_fits_w<float, PPM, 32, 8, 4>() && box_fits_w<float, PPM, 32, 15, 4>() &&
                  box_fits_w<float, PPM, 32, 8, 8>() && box_fits_w<double, PPM, 32, 8, 4>() &&
                  box_fits_w<double, PPM, 32, 15, 4>() && box_fits_w<double, PPM, 32, 8, 8>() &&
                  box_fits_w<float, WENO5, 32, 8, 8>() && box_fits_w<double, WENO5, 32, 8, 8>() &&
                  box_fits_w<float, WENO7, 32, 15, 4>() && box_fits_w<double, WENO7, 32, 15, 4>(),
              "axis-0 bulk-copy box exceeds the w level");

template <typename T, int SCH> bool check_scheme() {
  return check_all<T, SCH, 0, 32, 8>() && check_all<T, SCH, 1, 32, 8>() && check_all<T, SCH, 0, 32, 15>() &&
         check_all<T, SCH, 1, 32, 15>();
}

int main() {
  const bool ok = check_scheme<float, PCM>() && check_scheme<float, PLM>() && check_scheme<float, PPM>() &&
                  check_scheme<float, WENO3>() && check_scheme<float, WENO5>() && check_scheme<float, WENO7>() &&
                  check_scheme<double, PCM>() && check_scheme<double, PLM>() && check_scheme<double, PPM>() &&
                  check_scheme<double, WENO3>() && check_scheme<double, WENO5>() && check_scheme<double, WENO7>();
  if (!ok) return 1;
  std::printf("ok %lld\n", g_checked);
  return 0;
}
