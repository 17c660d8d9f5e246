// Palette generator (multiwave.cpp) on the host and the C ABI of the
// colouring step; the per-pixel colour runs on the GPU (colour.cu).
#include "colour.hpp"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <sstream>
#include <string>

#include "handle.hpp"

namespace nmg {

uint8_t clip_byte(float x) {
  if (!(x > 0.0f)) return 0;
  if (x >= 255.0f) return 255;
  return (uint8_t)(x + 0.5f);
}

Rgb interp_rgb(Rgb a, Rgb b, float t) {
  const float s = 1.0f - t;
  return Rgb{clip_byte(s * a.r + t * b.r), clip_byte(s * a.g + t * b.g),
             clip_byte(s * a.b + t * b.b), 0};
}

Rgb hsl_to_rgb(float h, float s, float l) {
  float hh = std::fmod(h, 360.0f);
  if (hh < 0.0f) hh += 360.0f;
  const float c = (1.0f - std::fabs(2.0f * l - 1.0f)) * s;
  const float hp = hh / 60.0f;
  const float x = c * (1.0f - std::fabs(std::fmod(hp, 2.0f) - 1.0f));
  float r = 0.0f, g = 0.0f, b = 0.0f;
  switch ((int)hp % 6) {
    case 0: r = c; g = x; break;
    case 1: r = x; g = c; break;
    case 2: g = c; b = x; break;
    case 3: g = x; b = c; break;
    case 4: r = x; b = c; break;
    default: r = c; b = x; break;
  }
  const float m = l - 0.5f * c;
  return Rgb{clip_byte(255.0f * (r + m)), clip_byte(255.0f * (g + m)), clip_byte(255.0f * (b + m)),
             0};
}

// Linear interpolation around the cycle of values, in double as the
// reference's (1.0 - t) promotes it (multiwave.cpp:5-12).
float FloatCycle::value(int step) const {
  const int n = (int)values.size();
  float t = n * (step % period) / (float)period;
  const int i0 = (int)t;
  const int i1 = (i0 + 1) % n;
  t -= i0;
  return (float)((1.0 - t) * values[i0] + t * values[i1]);
}

float FloatWave::value(int step) const {  // multiwave.cpp:14-17
  constexpr float kTau = 2.0 * 3.14159265358979;
  return amplitude * std::sin(step * kTau / period);
}

bool MultiWave::valid() const {
  if (hue_cycles.empty() || hue_period < 1 || sat_cycle.values.empty() || sat_cycle.period < 1)
    return false;
  for (const FloatCycle& c : hue_cycles)
    if (c.values.empty() || c.period < 1) return false;
  for (const FloatWave& w : lum_waves)
    if (w.period < 1) return false;
  return true;
}

// The reference's text format: number of hue cycles, each as (count, values,
// period); the hue period; the saturation cycle; the luminance waves as
// (amplitude, period) pairs.
bool MultiWave::load(const char* path) {
  FILE* fp = std::fopen(path, "r");
  if (!fp) return false;
  MultiWave w;
  int n = 0;
  bool ok = std::fscanf(fp, "%d", &n) == 1 && n > 0;
  if (ok) w.hue_cycles.resize(n);
  for (size_t i = 0; ok && i < w.hue_cycles.size(); i++) {
    int m = 0;
    ok = std::fscanf(fp, "%d", &m) == 1 && m > 0;
    if (!ok) break;
    w.hue_cycles[i].values.resize(m);
    for (int j = 0; ok && j < m; j++) ok = std::fscanf(fp, "%f", &w.hue_cycles[i].values[j]) == 1;
    ok = ok && std::fscanf(fp, "%d", &w.hue_cycles[i].period) == 1;
  }
  ok = ok && std::fscanf(fp, "%d", &w.hue_period) == 1;
  ok = ok && std::fscanf(fp, "%d", &n) == 1 && n > 0;
  if (ok) w.sat_cycle.values.resize(n);
  for (int j = 0; ok && j < n; j++) ok = std::fscanf(fp, "%f", &w.sat_cycle.values[j]) == 1;
  ok = ok && std::fscanf(fp, "%d", &w.sat_cycle.period) == 1;
  ok = ok && std::fscanf(fp, "%d", &n) == 1 && n >= 0;
  if (ok) w.lum_waves.resize(n);
  for (int j = 0; ok && j < n; j++)
    ok = std::fscanf(fp, "%f %d", &w.lum_waves[j].amplitude, &w.lum_waves[j].period) == 2;
  std::fclose(fp);
  if (!ok || !w.valid()) return false;
  *this = w;
  return true;
}

bool MultiWave::save(const char* path) const {
  FILE* fp = std::fopen(path, "w");
  if (!fp) return false;
  std::fprintf(fp, "%d\n", (int)hue_cycles.size());
  for (const FloatCycle& c : hue_cycles) {
    std::fprintf(fp, "%d ", (int)c.values.size());
    for (float v : c.values) std::fprintf(fp, "%f ", v);
    std::fprintf(fp, "%d\n", c.period);
  }
  std::fprintf(fp, "%d\n\n", hue_period);
  std::fprintf(fp, "%d\n", (int)sat_cycle.values.size());
  for (float v : sat_cycle.values) std::fprintf(fp, "%f ", v);
  std::fprintf(fp, "\n%d\n\n", sat_cycle.period);
  std::fprintf(fp, "%d\n", (int)lum_waves.size());
  for (const FloatWave& w : lum_waves) std::fprintf(fp, "%f %d\n", w.amplitude, w.period);
  return std::fclose(fp) == 0;
}

// multiwave.cpp:75-116: for each entry, saturation from its cycle, luminance
// from the logistic of the summed waves, and hue interpolated within and then
// between two neighbouring hue cycles.
std::vector<Rgb> MultiWave::cache(int n) const {
  std::vector<Rgb> pal((size_t)(n > 0 ? n : 0));
  const int ncyc = (int)hue_cycles.size();
  auto along = [&](const FloatCycle& cyc, int i, float sat, float lum) {
    const int m = (int)cyc.values.size();
    float tx = m * (i % cyc.period) / (float)cyc.period;
    const int x0 = (int)tx;
    const int x1 = (x0 + 1) % m;
    tx -= x0;
    return interp_rgb(hsl_to_rgb(cyc.values[x0], sat, lum), hsl_to_rgb(cyc.values[x1], sat, lum),
                      tx);
  };
  for (int i = 0; i < n; i++) {
    const float sat = sat_cycle.value(i);
    float lum = 0.0f;
    for (const FloatWave& w : lum_waves) lum += w.value(i);
    lum = (float)(1.0 / (1.0 + std::exp(-lum)));
    float ty = ncyc * (i % hue_period) / (float)hue_period;
    const int y0 = (int)ty;
    const int y1 = (y0 + 1) % ncyc;
    ty -= y0;
    const Rgb c0 = along(hue_cycles[y0], i, sat, lum);
    const Rgb c1 = along(hue_cycles[y1], i, sat, lum);
    pal[(size_t)i] = interp_rgb(c0, c1, ty);
  }
  return pal;
}

cudaError_t launch_colour(const EscapeValue* grid, int nr, int nc, int sc, int N,
                          const Rgb* pal, int smooth, uint8_t* out, cudaStream_t s);

}  // namespace nmg

struct nm_palette {
  nmg::MultiWave wave;
  int cached_n = -1;
  std::vector<nmg::Rgb> pal;
  nmg::DevBuf<nmg::Rgb> d_pal;
  bool uploaded = false;
  int device = -1;
};

using nmg::fail;

namespace {

int ensure_cache(nm_palette* p, int n) {
  if (p->cached_n == n) return NM_OK;
  p->pal = p->wave.cache(n);
  p->cached_n = n;
  p->uploaded = false;
  return NM_OK;
}

}  // namespace

extern "C" {

nm_palette* nm_palette_load(const char* path) {
  if (!path) {
    fail(NM_ERR_ARG, "null path");
    return nullptr;
  }
  std::unique_ptr<nm_palette> p(new nm_palette());
  if (!p->wave.load(path)) {
    fail(NM_ERR_IO, "cannot read a palette from %s", path);
    return nullptr;
  }
  return p.release();
}

int nm_palette_save(const nm_palette* p, const char* path) {
  if (!p || !path) return fail(NM_ERR_ARG, "null palette or path");
  if (!p->wave.save(path)) return fail(NM_ERR_IO, "cannot write %s", path);
  return NM_OK;
}

void nm_palette_destroy(nm_palette* p) { delete p; }

int nm_palette_cache(nm_palette* p, int n, unsigned char* rgb_out) {
  if (!p || !rgb_out || n < 0) return fail(NM_ERR_ARG, "palette cache arguments");
  if (int rc = ensure_cache(p, n)) return rc;
  for (int i = 0; i < n; i++) {
    rgb_out[3 * i] = p->pal[(size_t)i].r;
    rgb_out[3 * i + 1] = p->pal[(size_t)i].g;
    rgb_out[3 * i + 2] = p->pal[(size_t)i].b;
  }
  return NM_OK;
}

int nm_colorize(nm_handle* h, nm_palette* p, int sc, int smooth, unsigned char* rgb_out) {
  if (!h || !p || !rgb_out || sc < 1) return fail(NM_ERR_ARG, "colorize arguments");
  if (!h->stream || !h->grid.p) return fail(NM_ERR_STATE, "nothing rendered yet");
  const int nr = h->grid_nr, nc = h->grid_nc;
  if (nr % sc || nc % sc)
    return fail(NM_ERR_ARG, "grid %d x %d is not a multiple of %d", nr, nc, sc);
  const int N = h->view.iterations();
  if (int rc = ensure_cache(p, N)) return rc;
  if (!p->uploaded || p->device != h->device) {
    NM_CUDA(p->d_pal.reserve(p->pal.size()));
    if (!p->pal.empty())
      NM_CUDA(cudaMemcpyAsync(p->d_pal.p, p->pal.data(), p->pal.size() * sizeof(nmg::Rgb),
                              cudaMemcpyHostToDevice, h->stream));
    p->uploaded = true;
    p->device = h->device;
  }
  const size_t bytes = (size_t)(nr / sc) * (nc / sc) * 3;
  nmg::DevBuf<uint8_t> d_out;
  NM_CUDA(d_out.reserve(bytes));
  NM_CUDA(nmg::launch_colour(h->grid.p, nr, nc, sc, N, p->d_pal.p, smooth, d_out.p, h->stream));
  NM_CUDA(cudaMemcpyAsync(rgb_out, d_out.p, bytes, cudaMemcpyDeviceToHost, h->stream));
  NM_CUDA(cudaStreamSynchronize(h->stream));
  return NM_OK;
}

int nm_write_ppm(const char* path, const unsigned char* rgb, int rows, int cols) {
  if (!path || !rgb || rows < 1 || cols < 1) return fail(NM_ERR_ARG, "ppm arguments");
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return fail(NM_ERR_IO, "cannot write %s", path);
  std::fprintf(fp, "P6\n%d %d\n255\n", cols, rows);
  const size_t n = (size_t)rows * cols * 3;
  const bool ok = std::fwrite(rgb, 1, n, fp) == n;
  if (std::fclose(fp) != 0 || !ok) return fail(NM_ERR_IO, "cannot write %s", path);
  return NM_OK;
}

}  // extern "C"
