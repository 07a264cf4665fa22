// Detector-frame preparation: clipping and 2^n x 2^n binning of photon-count
// frames (spinifel/prep.py:37-125) in one pass on the device.
//
// The reference clips the high-resolution border (N_clipping) and then sums
// (or averages) 2 x 2 blocks N_binning times on the host.  Here one thread
// produces one binned pixel: it maps the binned pixel to its
// 2^N_binning x 2^N_binning block of the clipped panel, the clipped panel to
// the raw panel (the PnCCD four-panel and monolithic layouts of
// prep.py:88-112), and sums the block in int64 (exact for uint16 counts), so
// the result is exactly the reference's repeated 2 x 2 sums; the mean is the
// sum / 4^N_binning (exact: a power of two).
#include <algorithm>

#include "common.cuh"

namespace {

// raw (row, col) of clipped panel pixel (r, c): prep.py clipping()
__device__ __forceinline__ void clip_map(int n_panels, int panel, int sa, int sb, int ca, int cb,
                                         int r, int c, int *rr, int *rc) {
  if (n_panels == 4) {  // panels 0 and 2 keep the last columns, 1 and 3 the first
    *rr = sa - ca + r;
    *rc = (panel == 0 || panel == 2) ? sb - cb + c : c;
  } else {  // monolithic: the central region
    *rr = sa / 2 - ca / 2 + r;
    *rc = sb / 2 - cb / 2 + c;
  }
}

// one CTA per (frame, panel) plane at a time (grid-stride over planes);
// 32-bit index arithmetic within a plane
__global__ void k_bin_frames(const uint16_t *__restrict__ raw, int64_t n_img, int n_panels, int sa,
                             int sb, int ca, int cb, int nb, int mean, bool vec4,
                             float *__restrict__ out) {
  const int f = 1 << nb;
  const int oa = ca >> nb, ob = cb >> nb;
  const int per_plane = oa * ob;
  const int64_t planes = n_img * n_panels;
  const double inv = 1.0 / (double)((int64_t)f * f);
  for (int64_t pl = blockIdx.x; pl < planes; pl += gridDim.x) {
    const int panel = (int)(pl % n_panels);
    const uint16_t *src = raw + pl * (int64_t)sa * sb;
    float *dst = out + pl * (int64_t)per_plane;
    for (int q = threadIdx.x; q < per_plane; q += blockDim.x) {
      const int pr = q / ob, pc = q - pr * ob;
      int64_t s = 0;
      for (int dr = 0; dr < f; ++dr) {
        int rr, rc;
        clip_map(n_panels, panel, sa, sb, ca, cb, pr * f + dr, pc * f, &rr, &rc);
        const uint16_t *row = src + (int64_t)rr * sb + rc;
        if (vec4 && f == 4) {  // the block row as one 8-byte load (4 counts)
          const uint2 v = *reinterpret_cast<const uint2 *>(row);
          s += (v.x & 0xFFFFu) + (v.x >> 16) + (v.y & 0xFFFFu) + (v.y >> 16);
        } else {
          for (int dc = 0; dc < f; ++dc) s += row[dc];
        }
      }
      dst[q] = mean ? (float)((double)s * inv) : (float)s;
    }
  }
}

}  // namespace

extern "C" int spf_bin_frames_u16(const uint16_t *d_raw, int64_t n_img, int n_panels, int sa,
                                  int sb, int n_clip, int n_bin, int mean, float *d_out,
                                  void *stream) {
  SPF_REQUIRE(n_img >= 0 && sa > 0 && sb > 0 && n_clip >= 0 && n_bin >= 0 && n_clip < 16 &&
                  n_bin < 16,
              "spf_bin_frames_u16: bad sizes");
  SPF_REQUIRE(n_panels == 4 || n_panels == 1 || n_clip == 0,
              "spf_bin_frames_u16: clipping is defined for 1 or 4 panels (prep.py:98-112)");
  SPF_REQUIRE(n_panels >= 1, "spf_bin_frames_u16: n_panels < 1");
  // clipped panel size: sa / 2^n_clip (four panels) or 2 * sa / 2^(n_clip+1) (one panel)
  int ca = sa >> n_clip, cb = sb >> n_clip;
  if (n_panels == 1 && n_clip > 0) {
    ca = 2 * (sa >> (n_clip + 1));
    cb = 2 * (sb >> (n_clip + 1));
  }
  SPF_REQUIRE(ca > 0 && cb > 0 && (ca >> n_bin) > 0 && (cb >> n_bin) > 0,
              "spf_bin_frames_u16: nothing left after clipping and binning");
  SPF_REQUIRE(ca % (1 << n_bin) == 0 && cb % (1 << n_bin) == 0,
              "spf_bin_frames_u16: clipped panel %d x %d not divisible by 2^%d", ca, cb, n_bin);
  if (n_img == 0) return SPF_OK;
  SPF_REQUIRE(d_raw && d_out, "spf_bin_frames_u16: NULL pointer");
  // 4 x 4 blocks as 8-byte row loads when every block row starts on an
  // 8-byte boundary: an aligned base, row length and clipped column offsets
  // multiples of 4 pixels
  const int col0 = n_panels == 1 ? sb / 2 - cb / 2 : sb - cb;
  const bool vec4 = n_bin == 2 && ((uintptr_t)d_raw % 8) == 0 && sb % 4 == 0 && col0 % 4 == 0;
  const int64_t planes = n_img * n_panels;
  k_bin_frames<<<(unsigned)std::min<int64_t>(planes, (int64_t)spf::sm_count() * 16), 256, 0,
                 spf::as_stream(stream)>>>(d_raw, n_img, n_panels, sa, sb, ca, cb, n_bin, mean,
                                           vec4, d_out);
  return spf::check_launch("k_bin_frames");
}
