// Colouring of the grid (multiwave.cpp, viewer.cpp:89-124): the multi-wave
// palette generator, its cached palette, and the per-pixel colour.
//
// The reference takes HSL conversion, colour interpolation and byte clipping
// from libbyteimage (axnjaxn/byteimage, version not pinned by the reference's
// makefile, absent here).  They are restated from their standard definitions:
//   clip(x)            : x clamped to [0, 255], rounded half up, as a byte;
//   interp(a, b, t)    : per channel clip((1 - t) a + t b);
//   hsl2rgb(h, s, l)   : the standard HSL -> RGB map (h in degrees), each
//                        channel clip(255 x).
#pragma once

#include <cstdint>
#include <vector>

namespace nmg {

struct Rgb {
  uint8_t r, g, b, pad_;
};

struct FloatCycle {  // multiwave.cpp:5-12
  std::vector<float> values;
  int period = 1;
  float value(int step) const;
};
struct FloatWave {  // multiwave.cpp:14-17
  float amplitude = 1.0f;
  int period = 1;
  float value(int step) const;
};

struct MultiWave {  // multiwave.h:8-37
  std::vector<FloatCycle> hue_cycles;
  int hue_period = 1;
  FloatCycle sat_cycle;
  std::vector<FloatWave> lum_waves;

  bool load(const char* path);        // multiwave.cpp:19-50
  bool save(const char* path) const;  // multiwave.cpp:52-73
  bool valid() const;                 // every cycle non-empty, every period positive
  std::vector<Rgb> cache(int n) const;  // multiwave.cpp:75-116
};

uint8_t clip_byte(float x);
Rgb interp_rgb(Rgb a, Rgb b, float t);
Rgb hsl_to_rgb(float h, float s, float l);

}  // namespace nmg
