// render.cu -- Renderer::render (painty/renderer/Renderer.hxx:60-156): the canvas composed
// onto its substrate and lit by a point light, fused into one pass.
//
// Per pixel: the Kubelka-Munk composite of the wet layer over R0 (the diffuse colour Kd);
// a normal from central differences of the wet layer's volume (the height map, read at the
// four neighbours with BORDER_REFLECT, as painty's Interpolate at integer positions);
// Cook-Torrance shading with painty's Beckmann term exp(-tan^2(acos(NdotH)) / m^2) /
// (m^2 + NdotH^4 pi), geometric term min(1, 2 NdotH NdotV / VdotH, 2 NdotH NdotL / VdotH),
// Schlick Fresnel with Ks = 1, light (-200, -1500, -2000) of power 15, eye over the canvas
// centre at z = -100, roughness 0.5, specular share 0.2, ambient 0.2 Kd^2; clamped to [0, 1].
// F64 canvases compute in double with painty's expressions and operation order (sums left to
// right, normalisation by division by sqrt of the squared norm, the same libm functions).
// F32 / F16 / BF16 canvases compute in float with closed forms of the same terms (reciprocal
// square roots, tan^2(acos x) = (1 - x^2) / x^2, Fresnel 1 for Ks = 1). One pass reads each
// pixel record once (neighbour volumes come from the same lines in L1/L2) and writes the three
// output planes.
#include "device_common.cuh"
#include "internal.h"

namespace pg {
namespace {

template <class M>
struct V3 {
  M x, y, z;
};
template <class M>
__device__ __forceinline__ M dot3(V3<M> a, V3<M> b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <class M>
__device__ __forceinline__ V3<M> nrm3(V3<M> a) {
  const M n = dot3(a, a);
  if (n > M(0)) {
    if constexpr (sizeof(M) == 8) {
      const M r = sqrt(n);
      return {a.x / r, a.y / r, a.z / r};
    } else {
      const M k = rsqrtf(n);
      return {a.x * k, a.y * k, a.z * k};
    }
  }
  return a;
}
__device__ __forceinline__ int reflect_edge(int p, int n) {  // BORDER_REFLECT one step out
  return p < 0 ? 0 : (p >= n ? n - 1 : p);
}

template <class TK, class TV, class M, class TR>
__global__ void __launch_bounds__(256) render_lit_kernel(const void* canvas, const TR* r0_0,
                                                         const TR* r0_1, const TR* r0_2,
                                                         TR* o0, TR* o1, TR* o2, int rows,
                                                         int cols, int64_t pitch) {
  const int j = blockIdx.x * 32 + threadIdx.x;
  const int i = blockIdx.y * 8 + threadIdx.y;
  if (i >= rows || j >= cols) return;
  const int64_t p = static_cast<int64_t>(i) * pitch + j;
  const PixRec<TK, TV> r = load_rec<false, TK, TV>(canvas, static_cast<int>(p));
  auto vol = [&](int y, int x) {
    return ld_elem<M>(rec_v<TK, TV>(const_cast<void*>(canvas),
                                    static_cast<int>(static_cast<int64_t>(y) * pitch + x)));
  };
  const M s11 = ld_elem<M>(&r.v[6]);
  const M s01 = vol(i, reflect_edge(j - 1, cols)), s21 = vol(i, reflect_edge(j + 1, cols));
  const M s10 = vol(reflect_edge(i - 1, rows), j), s12 = vol(reflect_edge(i + 1, rows), j);
  // the composite (Renderer::compose)
  const TR r0[3] = {r0_0[p], r0_1[p], r0_2[p]};
  M Kd[3];
#pragma unroll
  for (int c = 0; c < 3; c++)
    Kd[c] = km_reflectance(ld_elem<M>(&r.k[c]), ld_elem<M>(&r.k[3 + c]), static_cast<M>(r0[c]), s11);
  // normal from the height map (Renderer.hxx:103-119)
  const V3<M> va = nrm3<M>({M(2), M(0), s21 - s01});
  const V3<M> vb = nrm3<M>({M(0), M(2), s12 - s10});
  V3<M> n = nrm3<M>({va.y * vb.z - va.z * vb.y, va.z * vb.x - va.x * vb.z, va.x * vb.y - va.y * vb.x});
  n.z *= M(-1);
  const M fj = static_cast<M>(j), fi = static_cast<M>(i);
  const V3<M> lightDirection = nrm3<M>({M(-200) - fj, M(-1500) - fi, M(-2000.) - s11});
  const V3<M> l = nrm3(lightDirection);
  // eyePos = (width / 2.0, height / 2.0, -100): exact in float too (sizes below 2^24)
  const V3<M> v = nrm3<M>({static_cast<M>(cols) * M(0.5) - fj, static_cast<M>(rows) * M(0.5) - fi,
                           M(-100.) - s11});
  const V3<M> h = nrm3<M>({v.x + l.x, v.y + l.y, v.z + l.z});
  const M NdotH = fmax(M(0), dot3(n, h));
  const M VdotH = fmax(M(0), dot3(v, h));
  const M NdotV = fmax(M(0), dot3(n, v));
  const M NdotL = fmax(M(0), dot3(n, l));
  constexpr M Pi = M(3.141592653589793238462643383279502884);
  const M m = M(0.5), s = M(0.2);
  M spec = M(0);
  M beta;
  if constexpr (sizeof(M) == 8) {  // painty's expressions, function for function
    if (NdotL > M(0) && NdotV > M(0)) {
      const M A = M(1) / (pow(m, M(2)) + pow(NdotH, M(4)) * Pi);
      const M B = exp(-pow(tan(acos(NdotH)), M(2)) / pow(m, M(2)));
      const M G1 = M(2) * NdotH * NdotV / VdotH;
      const M G2 = M(2) * NdotH * NdotL / VdotH;
      const M gmin = G2 < G1 ? G2 : G1;  // std::min(G1, G2)
      const M G = gmin < M(1) ? gmin : M(1);
      const M RF = M(1) + (M(1) - M(1)) * pow(M(1) - VdotH, M(5));  // Ks = 1
      spec = A * B * G * RF / (NdotL * NdotV);
    }
    beta = M(15) * (M(1) / (M(4) * Pi * pow(sqrt(dot3(lightDirection, lightDirection)), M(2))));
  } else {
    // the same terms in closed form: tan^2(acos x) = (1 - x^2) / x^2, m^2 = 1/4, Fresnel with
    // Ks = 1 is 1, |lightDirection|^2 for the squared norm of the sqrt
    if (NdotL > 0.0f && NdotV > 0.0f) {
      const float c2 = NdotH * NdotH;
      const float A = 1.0f / (0.25f + c2 * c2 * Pi);
      const float B = __expf(-4.0f * (1.0f - c2) / c2);
      const float G = fminf(1.0f, 2.0f * NdotH * fminf(NdotV, NdotL) / VdotH);
      spec = A * B * G / (NdotL * NdotV);
    }
    beta = 15.0f / (4.0f * Pi * dot3(lightDirection, lightDirection));
  }
  TR* out[3] = {o0, o1, o2};
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const M ambient = Kd[c] * M(0.2);
    const M res = (beta * NdotL) * ((M(1) - s) * Kd[c] + s * spec) + ambient * Kd[c];
    const M lo = res < M(0) ? M(0) : res;  // std::max(res, 0)
    out[c][p] = static_cast<TR>(M(1) < lo ? M(1) : lo);
  }
}

template <class TK, class TV, class M, class TR>
void launch_render(const painty_canvas* c, painty_image* out, cudaStream_t st) {
  const dim3 block(32, 8);
  const dim3 grid((c->wet.cols + 31) / 32, (c->wet.rows + 7) / 8);
  render_lit_kernel<TK, TV, M, TR><<<grid, block, 0, st>>>(
    c->wet.base, static_cast<const TR*>(c->r0.R[0]), static_cast<const TR*>(c->r0.R[1]),
    static_cast<const TR*>(c->r0.R[2]), static_cast<TR*>(out->R[0]), static_cast<TR*>(out->R[1]),
    static_cast<TR*>(out->R[2]), c->wet.rows, c->wet.cols, c->wet.pitch);
  count_launch();
  PG_CUDA(cudaGetLastError());
}

}  // namespace
}  // namespace pg

using pg::guard;

extern "C" {

painty_status painty_canvas_render(const painty_canvas* c, painty_image* out, void* stream) {
  return guard([&] {
    PG_REQUIRE(c && out, "null handle");
    PG_REQUIRE(out->rows == c->wet.rows && out->cols == c->wet.cols, "image size differs");
    PG_REQUIRE(out->storage == c->r0.storage,
               "render into an F64 image for F64 canvases, an F32 image otherwise");
    PG_REQUIRE(static_cast<int64_t>(c->wet.rows) * c->wet.pitch < (int64_t(1) << 31),
               "canvas too large");
    const cudaStream_t st = pg::as_stream(stream);
    switch (c->wet.storage) {
      case PAINTY_STORAGE_F32: pg::launch_render<float, float, float, float>(c, out, st); break;
      case PAINTY_STORAGE_F16: pg::launch_render<__half, __half, float, float>(c, out, st); break;
      case PAINTY_STORAGE_BF16:
        pg::launch_render<__nv_bfloat16, __half, float, float>(c, out, st);
        break;
      case PAINTY_STORAGE_F64:
        pg::launch_render<double, double, double, double>(c, out, st);
        break;
    }
  });
}

}  // extern "C"
