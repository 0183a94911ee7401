/* ORACLE / TEST INFRASTRUCTURE ONLY.
 * Headless stand-in for the few SDL names the reference simulation uses
 * (ARD-simulator-190113/simulation.h:5,35 and simulation.cpp:323,362,366,409,413).
 * No window, renderer or graphics library is involved: the pixel buffer the
 * reference fills each step is plain host memory and is never shown. */
#pragma once
#include <cstdint>

typedef uint8_t Uint8;
typedef uint32_t Uint32;

typedef struct SDL_PixelFormat { Uint32 format; } SDL_PixelFormat;

#define SDL_PIXELFORMAT_RGBA8888 0x16462004u

/* The reference allocates a format every step and never frees it; returning a
 * per-thread static object keeps the headless run from leaking. */
static inline SDL_PixelFormat* SDL_AllocFormat(Uint32 format) {
  static thread_local SDL_PixelFormat f;
  f.format = format;
  return &f;
}

static inline Uint32 SDL_MapRGBA(const SDL_PixelFormat*, Uint8 r, Uint8 g, Uint8 b, Uint8 a) {
  return ((Uint32)r << 24) | ((Uint32)g << 16) | ((Uint32)b << 8) | (Uint32)a;
}
