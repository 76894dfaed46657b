// libmisc.h - host stand-ins for the Cell SPU intrinsics and MFC DMA calls
// cell/spu/trace_spu.cpp uses, after the Cell SDK documentation: 4-float
// and 4-uint vectors (`vector float` as a GCC vector type), spu_splats,
// spu_cmpgt (all-ones lanes where a > b), spu_sel (bitwise: pattern bit 0
// takes a, 1 takes b); a DMA get/put is a memcpy between the SPU-local
// buffer and the 32-bit effective address, which the harness maps back to
// the host pool (yvref_ea_to_ptr).
#pragma once
#include <cstring>

typedef float yvref_v4f __attribute__((vector_size(16)));
typedef unsigned int yvref_v4u __attribute__((vector_size(16)));

inline yvref_v4f spu_splats(float x) {
  yvref_v4f r = {x, x, x, x};
  return r;
}
inline yvref_v4u spu_cmpgt(yvref_v4f a, yvref_v4f b) {
  yvref_v4u r;
  for (int i = 0; i < 4; ++i) r[i] = a[i] > b[i] ? 0xFFFFFFFFu : 0u;
  return r;
}
inline yvref_v4f spu_sel(yvref_v4f a, yvref_v4f b, yvref_v4u pattern) {
  yvref_v4u ua, ub;
  std::memcpy(&ua, &a, 16);
  std::memcpy(&ub, &b, 16);
  const yvref_v4u r = (ua & ~pattern) | (ub & pattern);
  yvref_v4f out;
  std::memcpy(&out, &r, 16);
  return out;
}

#define MFC_GET_CMD 0x40
#define MFC_PUT_CMD 0x20
#define MFC_TAG_UPDATE_ALL 2
#define MFC_WrTagMask 22

extern "C" void* yvref_ea_to_ptr(unsigned int ea);
inline void spu_mfcdma32(void* ls, unsigned int ea, unsigned int size, unsigned int,
                         unsigned int cmd) {
  if (cmd == MFC_GET_CMD)
    std::memcpy(ls, yvref_ea_to_ptr(ea), size);
  else
    std::memcpy(yvref_ea_to_ptr(ea), ls, size);
}
inline unsigned int spu_mfcstat(unsigned int) { return 0; }
inline unsigned int mfc_tag_reserve() { return 0; }
inline void spu_writech(int, int) {}

// `vector float` / `vector unsigned int` of the SPU language extensions
#define vector __attribute__((vector_size(16)))
