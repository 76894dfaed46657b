// ref_march_glue.cpp - compiles the reference's brick-skipping volume
// ray-march (reaction/trace/trace.cu with its utils.h, found on the include
// path that oracle/build_ref.py sets) on the host, with the stand-ins of
// ref_shim/cutil_math.h, and exposes castRay over a volume texture and a
// brick-mark texture.  Test infrastructure for oracle/_ref only.
#include "cutil_math.h"
#include "trace.cu"

uint3 threadIdx, blockIdx, blockDim;

// Composited RGBA of the rays from `eye` along the unit directions `dirs`
// (n x 3) through the volume (nx x ny x nz uint8, x fastest, normalized
// coordinates over [0, 1]^3) and the 64^3 brick marks.
extern "C" int yvref_cast_rays(const unsigned char* vol, int nx, int ny, int nz,
                               const unsigned char* marks, const float eye[3],
                               const float* dirs, int n, float* rgba) {
  volumeTex.data = vol;
  volumeTex.nx = nx;
  volumeTex.ny = ny;
  volumeTex.nz = nz;
  markTex.data = marks;
  markTex.nx = markTex.ny = markTex.nz = 64;
  c_eyePos = make_float3(eye[0], eye[1], eye[2]);
  for (int i = 0; i < n; ++i) {
    RayData r;
    r.orig = c_eyePos;
    r.dir = make_float3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]);
    const float4 c = castRay(r);
    rgba[4 * i] = c.x;
    rgba[4 * i + 1] = c.y;
    rgba[4 * i + 2] = c.z;
    rgba[4 * i + 3] = c.w;
  }
  return 0;
}
