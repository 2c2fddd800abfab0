// Device vertex / fragment shaders: the reference's software shaders as device functions.
//
//   Basic        Shader/Software/BasicSoft.h:62-79
//   Blinn-Phong  Shader/Software/BlinnPhongSoft.h:181-325 (point light, shininess 128, PCF shadow)
//   PBR + IBL    Shader/Software/PbrSoft.h:106-323
//   Blinn-Phong directional (shininess 32) and vertex colour: device shaders of the synthetic
//   benchmark scenes (no reference counterpart).
//
// Uniform bytes use the reference's ShaderUniforms layout (GLM aligned: vec3 = 16 B):
// UniformsModel @0 (reverseZ, model @16, MVP @80, inverse-transpose model mat3 @144,
// shadow MVP @192); Blinn-Phong/PBR: UniformsScene @256, UniformsMaterial @320;
// Basic/vertex colour: UniformsMaterial @256. Varyings are ShaderVaryings floats.
#pragma once

#include "sglc_device.cuh"

namespace sglc {

// Uniform reads. U = the draw's ShaderUniforms bytes (DrawParams::u) or, in a batched draw, the
// view's copy of them.
__device__ __forceinline__ const float *uMVP(const uint8_t *U) { return reinterpret_cast<const float *>(U + 80); }
__device__ __forceinline__ const float *uModel(const uint8_t *U) { return reinterpret_cast<const float *>(U + 16); }
__device__ __forceinline__ const float *uITModel(const uint8_t *U) { return reinterpret_cast<const float *>(U + 144); }
__device__ __forceinline__ const float *uShadowMVP(const uint8_t *U) { return reinterpret_cast<const float *>(U + 192); }
__device__ __forceinline__ int uI32(const uint8_t *U, int off) { return *reinterpret_cast<const int32_t *>(U + off); }
__device__ __forceinline__ float uF32(const uint8_t *U, int off) { return *reinterpret_cast<const float *>(U + off); }
__device__ __forceinline__ float4 uV4(const uint8_t *U, int off) { return *reinterpret_cast<const float4 *>(U + off); }

// VS: writes clip position and the varyings of one vertex. a = raw attribute floats.
template<int SH>
__device__ __forceinline__ float4 runVS(const DrawParams &p, const uint8_t *U, const float *a, float *v) {
  float4 position = make_float4(a[0], a[1], a[2], 1.0f);
  float4 pos = mul44(uMVP(U), position);
  if (SH == SH_FXAA) {   // FxaaSoft.h:60-63: the quad is already in clip space
    pos = position;
    v[0] = a[4];
    v[1] = a[5];
  } else if (SH == SH_SKYBOX || SH == SH_IBL_IRR || SH == SH_IBL_PRE) {
    // SkyboxSoft.h:67-76 (x, y, w, w; z = 0 with reversed Z), IBL*Soft.h VS (z = w): the cube sits
    // on the far plane
    if (SH == SH_SKYBOX) pos = make_float4(pos.x, pos.y, pos.w, pos.w);
    else pos.z = pos.w;
    if (SH == SH_SKYBOX && uI32(U, 0)) pos.z = 0.f;
    v[0] = a[0]; v[1] = a[1]; v[2] = a[2];
  } else if (SH == SH_VCOLOR) {
    v[0] = a[4]; v[1] = a[5]; v[2] = a[6]; v[3] = a[7];
  } else if (SH == SH_BLINN || SH == SH_BLINN_DIR || SH == SH_PBR) {
    const bool bp = SH != SH_PBR;
    v[0] = a[4];
    v[1] = a[5];
    if (bp) {
      float4 s = mul44(uShadowMVP(U), position);
      v[20] = s.x; v[21] = s.y; v[22] = s.z; v[23] = s.w;
    }
    float4 w4 = mul44(uModel(U), position);
    f3 world = mk3(w4.x, w4.y, w4.z);
    f3 nvec = mul33(uModel(U), mk3(a[8], a[9], a[10]));
    f3 lpos = ld3(U + 288);
    f3 ldir = (SH == SH_BLINN_DIR) ? lpos : lpos - world;
    f3 cdir = ld3(U + 272) - world;
    v[4] = nvec.x; v[5] = nvec.y; v[6] = nvec.z;
    v[8] = world.x; v[9] = world.y; v[10] = world.z;
    v[12] = cdir.x; v[13] = cdir.y; v[14] = cdir.z;
    v[16] = ldir.x; v[17] = ldir.y; v[18] = ldir.z;
    if (p.def[1]) {   // NORMAL_MAP
      f3 N = normalize3(mul33(uITModel(U), mk3(a[8], a[9], a[10])));
      f3 T = normalize3(mul33(uITModel(U), mk3(a[12], a[13], a[14])));
      f3 Tn = normalize3(T - dot3(T, N) * N);
      const int o = bp ? 24 : 20;
      v[o] = N.x; v[o + 1] = N.y; v[o + 2] = N.z;
      v[o + 4] = Tn.x; v[o + 5] = Tn.y; v[o + 6] = Tn.z;
    }
  }
  return pos;
}

// Interpolated varyings of one fragment, evaluated on demand from the triangle's three vertex
// rows with the reference's AVX2 sequence: s = v0*b0; s = fma(v1,b1,s); s = fma(v2,b2,s).
struct Vary {
  const float *r0, *r1, *r2;
  float b0, b1, b2;
  __device__ __forceinline__ float operator[](int i) const {
    float s = __ldg(r0 + i) * b0;
    s = __fmaf_rn(__ldg(r1 + i), b1, s);
    s = __fmaf_rn(__ldg(r2 + i), b2, s);
    return s;
  }
  __device__ __forceinline__ f3 v3(int i) const { return mk3((*this)[i], (*this)[i + 1], (*this)[i + 2]); }
};

struct FragIn {
  const uint8_t *U;   // uniforms
  Vary v;
  float dudx, dvdx, dudy, dvdy;   // texcoord differences p1-p0, p2-p0 of the quad
};

// ShaderSoft::getSampler2DLod (Render/Software/ShaderSoft.h:117-133)
__device__ __forceinline__ float lodOf(const DevSampler &s, const FragIn &f) {
  float tw = (float) s.width, th = (float) s.height;
  float dxx = f.dudx * tw, dxy = f.dvdx * th;
  float dyx = f.dudy * tw, dyy = f.dvdy * th;
  float d = gmax(dxx * dxx + dxy * dxy, dyx * dyx + dyy * dyy);
  return gmax(0.5f * log2f(d), 0.0f);
}

// ShaderSoft::texture for RGBA8 2D samplers: texel / 255
__device__ __forceinline__ float4 tex2D(const DrawParams &p, int slot, float u, float v, const FragIn &f) {
  const DevSampler &s = p.samp[slot];
  float lod = 0.f;
  if (s.lodFromDerivative) lod += lodOf(s, f);
  const float4 c = textureRGBA8(s, 0, u, v, lod);
  return make_float4(div255(c.x), div255(c.y), div255(c.z), div255(c.w));
}

__device__ __forceinline__ float4 texCube(const DrawParams &p, int slot, f3 d, float lod) {
  int face;
  float u, v;
  cubeUV(d, &face, &u, &v);
  const float4 c = textureRGBA8(p.samp[slot], face, u, v, lod);
  return make_float4(div255(c.x), div255(c.y), div255(c.z), div255(c.w));
}

__device__ __forceinline__ f3 normalFromMap(const DrawParams &p, const FragIn &f, int nOff, int tOff) {
  if (p.def[1]) {
    f3 N = normalize3(f.v.v3(nOff));
    f3 T = normalize3(f.v.v3(tOff));
    T = normalize3(T - dot3(T, N) * N);
    f3 B = cross3(T, N);
    float4 t = tex2D(p, 1, f.v[0], f.v[1], f);
    f3 tn = mk3(t.x * 2.0f - 1.0f, t.y * 2.0f - 1.0f, t.z * 2.0f - 1.0f);
    f3 r = mk3(T.x * tn.x + B.x * tn.y + N.x * tn.z, T.y * tn.x + B.y * tn.y + N.y * tn.z,
               T.z * tn.x + B.z * tn.y + N.z * tn.z);
    return normalize3(r);
  }
  return normalize3(f.v.v3(4));
}

// BlinnPhongSoft.h:247-271 (3x3 PCF against a FLOAT32 shadow map, sampler slot 4)
__device__ inline float shadowCalc(const DrawParams &p, const FragIn &f, f3 normal) {
  float fx = f.v[20], fy = f.v[21], fz = f.v[22], fw = f.v[23];
  float px = fx / fw, py = fy / fw, cur = fz / fw;
  if (cur < 0.f || cur > 1.f) return 0.0f;
  float bias = gmax(0.00025f * (1.0f - dot3(normal, normalize3(f.v.v3(16)))), 0.00005f);
  const DevSampler &s = p.samp[4];
  float ox = 1.0f / (float) s.tex.w[0], oy = 1.0f / (float) s.tex.h[0];
  int reverseZ = uI32(f.U, 0);
  float shadow = 0.0f;
  // a NEAREST shadow map is read at level 0 whatever the LOD: the nine taps inline the nearest
  // lookup (the same arithmetic as textureImpl's) instead of nine sampler calls
  const bool nearest0 = s.filter == FILTER_NEAREST && s.tex.levels > 0;
  for (int x = -1; x <= 1; ++x)
    for (int y = -1; y <= 1; ++y) {
      const float u = px + (float) x * ox, v = py + (float) y * oy;
      float pcf = nearest0 ? __uint_as_float(nearestSample(s.tex, 0, 0, u, v, s.wrap, s.border))
                           : __uint_as_float(textureImpl(s, 0, u, v, 0.f));
      if (reverseZ) shadow += cur + bias < pcf ? 1.0f : 0.0f;
      else shadow += cur - bias > pcf ? 1.0f : 0.0f;
    }
  return shadow / 9.0f;
}

template<bool DIRECTIONAL>
__device__ inline float4 fsBlinnPhong(const DrawParams &p, const FragIn &f) {
  const float specExp = DIRECTIONAL ? 32.f : 128.f;
  const float rangeInv = 1.0f / 5.f;
  float4 base = p.def[0] ? tex2D(p, 0, f.v[0], f.v[1], f) : uV4(f.U, 352);
  f3 N = normalFromMap(p, f, 24, 28);
  float ao = 1.f;
  if (p.def[3]) ao = tex2D(p, 3, f.v[0], f.v[1], f).x;
  f3 baseRgb = mk3(base.x, base.y, base.z);
  f3 ambient = baseRgb * ld3(f.U + 256) * ao;
  f3 diffuseC = mk3(0, 0, 0), specC = mk3(0, 0, 0), emis = mk3(0, 0, 0);
  if (uI32(f.U, 320)) {
    f3 ldirRaw = f.v.v3(16);
    f3 lightColor = ld3(f.U + 304);
    f3 L = normalize3(ldirRaw);
    float diffuse = gmax(dot3(N, L), 0.0f);
    if (DIRECTIONAL) {
      diffuseC = lightColor * baseRgb * diffuse;
    } else {
      f3 lDir = ldirRaw * rangeInv;
      float att = gclamp(1.0f - dot3(lDir, lDir), 0.0f, 1.0f);
      diffuseC = lightColor * baseRgb * diffuse * att;
    }
    f3 C = normalize3(f.v.v3(12));
    f3 H = normalize3(L + C);
    float sa = gmax(dot3(N, H), 0.0f);
    float pw = powf(sa, specExp);
    specC = uF32(f.U, 336) * mk3(pw, pw, pw);
    if (uI32(f.U, 328)) {
      float shadow = 1.0f - shadowCalc(p, f, N);
      diffuseC = diffuseC * shadow;
      specC = specC * shadow;
    }
  }
  if (p.def[2]) {
    float4 e = tex2D(p, 2, f.v[0], f.v[1], f);
    emis = mk3(e.x, e.y, e.z);
  }
  f3 c = ambient + diffuseC + specC + emis;
  return make_float4(c.x, c.y, c.z, base.w);
}

// Training record of the neural IBL shader (sglc_nn.cuh): the network's 12 inputs and the square
// root of the IBL term it learns, appended while the host has capture enabled.
static __device__ __forceinline__ void captureRecord(const DrawParams &p, f3 N, f3 V, float roughness, float metallic,
                                           float4 albedo, float NdotV, f3 ibl) {
  unsigned long long slot = atomicAdd(p.capCount, 1ull);
  if (slot % (unsigned) p.capStride) return;
  slot /= (unsigned) p.capStride;
  if (slot >= (unsigned long long) p.capCap) return;
  float4 *r = reinterpret_cast<float4 *>(p.capRecords + slot * 16);
  r[0] = make_float4(N.x, N.y, N.z, V.x);
  r[1] = make_float4(V.y, V.z, roughness, metallic);
  r[2] = make_float4(albedo.x, albedo.y, albedo.z, NdotV);
  r[3] = make_float4(sqrtf(fmaxf(ibl.x, 0.f)), sqrtf(fmaxf(ibl.y, 0.f)), sqrtf(fmaxf(ibl.z, 0.f)), 0.f);
}

// The PBR fragment shader's surface terms (PbrSoft.h:229-294): material texels, the normal-mapped
// normal, the view direction, the direct point light and the emissive texel.
struct PbrSurface {
  float4 arg;          // albedo texel (or base colour)
  f3 albedo;           // linear albedo
  float metallic, roughness, ao;
  f3 N, V, F0, Lo;
  f3 emissive;
};

// EMISSIVE: also fetch the emissive texel here (the neural variant finishes the colour later, when
// the fragment inputs are gone); the plain shader fetches it at the end, as PbrSoft.h:315-318 does.
template<bool EMISSIVE>
__device__ __forceinline__ PbrSurface pbrSurface(const DrawParams &p, const FragIn &f) {
  const float PI = 3.14159265359f;
  const float rangeInv = 1.0f / 5.f;
  PbrSurface s;
  float4 arg = p.def[0] ? tex2D(p, 0, f.v[0], f.v[1], f) : uV4(f.U, 352);
  s.arg = arg;
  // The PBR shader's powers (albedo linearisation, Fresnel (1 - cos)^5, gamma) use the special-
  // function pow (exp2(y log2 x), a few ulp for these exponents and bases in [0, 1]): an error of a
  // few ulp moves a colour across a u8 boundary in about one channel in 10^4, by one step. Measured
  // on GB300 against the oracle: the 1080p MSAA4 frame keeps 0.999987 of its pixels within 1 LSB
  // (as with powf), and k_shade drops from 0.129 to 0.117 ms.
  f3 albedo = mk3(__powf(arg.x, 2.2f), __powf(arg.y, 2.2f), __powf(arg.z, 2.2f));
  s.albedo = albedo;
  float metallic = 0.0f, roughness = 1.0f;
  if (p.def[4]) {
    float4 mr = tex2D(p, 4, f.v[0], f.v[1], f);
    metallic = mr.z;
    roughness = mr.y;
  }
  s.metallic = metallic;
  s.roughness = roughness;
  float ao = 1.f;
  if (p.def[3]) ao = tex2D(p, 3, f.v[0], f.v[1], f).x;
  s.ao = ao;
  f3 N = normalFromMap(p, f, 20, 24);
  f3 V = normalize3(f.v.v3(12));
  s.N = N;
  s.V = V;
  f3 F0 = mk3(0.04f, 0.04f, 0.04f);
  F0 = F0 * (1.0f - metallic) + albedo * metallic;
  s.F0 = F0;
  f3 Lo = mk3(0, 0, 0);
  if (uI32(f.U, 320)) {
    f3 ldir = f.v.v3(16);
    f3 L = normalize3(ldir);
    f3 H = normalize3(V + L);
    f3 lDir = ldir * rangeInv;
    float att = gclamp(1.0f - dot3(lDir, lDir), 0.0f, 1.0f);
    f3 radiance = ld3(f.U + 304) * att;
    float a = roughness * roughness;
    float a2 = a * a;
    float NdotH = gmax(dot3(N, H), 0.0f);
    float NdotH2 = NdotH * NdotH;
    float denom = (NdotH2 * (a2 - 1.0f) + 1.0f);
    denom = PI * denom * denom;
    float NDF = a2 / denom;
    float NdotV = gmax(dot3(N, V), 0.0f);
    float NdotL = gmax(dot3(N, L), 0.0f);
    float r1 = (roughness + 1.0f);
    float k = (r1 * r1) / 8.0f;
    float ggx2 = NdotV / (NdotV * (1.0f - k) + k);
    float ggx1 = NdotL / (NdotL * (1.0f - k) + k);
    float G = ggx1 * ggx2;
    float ct = gmax(dot3(H, V), 0.0f);
    float p5 = __powf(gclamp(1.0f - ct, 0.0f, 1.0f), 5.0f);
    f3 F = F0 + (1.0f - F0) * p5;
    f3 numerator = NDF * G * F;
    float denominator = 4.0f * gmax(dot3(N, V), 0.0f) * gmax(dot3(N, L), 0.0f) + 0.0001f;
    f3 specular = numerator / denominator;
    f3 kD = 1.0f - F;
    kD = kD * (1.0f - metallic);
    float NdL = gmax(dot3(N, L), 0.0f);
    Lo = Lo + (kD * albedo / PI + specular) * radiance * NdL;
  }
  s.Lo = Lo;
  s.emissive = mk3(0.f, 0.f, 0.f);
  if (EMISSIVE && p.def[2]) {
    float4 e = tex2D(p, 2, f.v[0], f.v[1], f);
    s.emissive = mk3(e.x, e.y, e.z);
  }
  return s;
}

// gamma correction and emissive (PbrSoft.h:311-321)
__device__ __forceinline__ float4 pbrFinish(const DrawParams &p, f3 ambient, f3 Lo, f3 emissive, float alpha) {
  f3 color = ambient + Lo;
  color = mk3(__powf(color.x, 1.0f / 2.2f), __powf(color.y, 1.0f / 2.2f), __powf(color.z, 1.0f / 2.2f));
  if (p.def[2]) color = color + emissive;
  return make_float4(color.x, color.y, color.z, alpha);
}

template<bool CAPTURE>
__device__ inline float4 fsPbr(const DrawParams &p, const FragIn &f) {
  PbrSurface s = pbrSurface<false>(p, f);
  const f3 N = s.N, V = s.V, F0 = s.F0, albedo = s.albedo;
  const float metallic = s.metallic, roughness = s.roughness, ao = s.ao;
  f3 ambient;
  if (uI32(f.U, 324)) {
    f3 mV = -V;
    f3 R = mV - N * dot3(N, mV) * 2.0f;
    float NdotV = gmax(dot3(N, V), 0.0f);
    float p5 = __powf(gclamp(1.0f - NdotV, 0.0f, 1.0f), 5.0f);
    float omr = 1.0f - roughness;
    f3 F = F0 + (max3(mk3(omr, omr, omr), F0) - F0) * p5;
    f3 kD = 1.0f - F;
    kD = kD * (1.0f - metallic);
    float4 irr = texCube(p, 5, N, 0.f);
    f3 diffuse = mk3(irr.x, irr.y, irr.z) * albedo;
    float4 pre = texCube(p, 6, R, roughness * 4.0f);
    // EnvBRDFApprox (PbrSoft.h:209-223)
    float rx = roughness * -1.f + 1.f, ry = roughness * -0.0275f + 0.0425f;
    float rz = roughness * -0.572f + 1.04f, rw = roughness * 0.022f + -0.04f;
    float a004 = gmin(rx * rx, exp2f(-9.28f * NdotV)) * rx + ry;
    float ABx = -1.04f * a004 + rz;
    float ABy = 1.04f * a004 + rw;
    ABy *= gmax(0.f, gmin(1.f, 50.0f * F.y));
    f3 env = F * ABx + ABy;
    f3 specular = mk3(pre.x, pre.y, pre.z) * env;
    f3 ibl = kD * diffuse + specular;
    if (CAPTURE) captureRecord(p, N, V, roughness, metallic, s.arg, NdotV, ibl);
    ambient = ibl * ao;
  } else {
    ambient = ld3(f.U + 256) * albedo * ao;
  }
  f3 emissive = mk3(0.f, 0.f, 0.f);
  if (p.def[2]) {
    float4 e = tex2D(p, 2, f.v[0], f.v[1], f);
    emissive = mk3(e.x, e.y, e.z);
  }
  return pbrFinish(p, ambient, s.Lo, emissive, s.arg.w);
}

// ---- environment shaders (IBLGenerator's cube-face passes, Environment.cpp:152-195) ------------
// SkyboxSoft.h:84-103
__device__ inline float4 fsSkybox(const DrawParams &p, const FragIn &f) {
  f3 wp = f.v.v3(0);
  if (p.def[0]) {   // EQUIRECTANGULAR_MAP: SampleSphericalMap
    f3 dir = normalize3(wp);
    float u = atan2f(dir.z, dir.x), v = asinf(-dir.y);
    u = u * 0.1591f + 0.5f;
    v = v * 0.3183f + 0.5f;
    return tex2D(p, 0, u, v, f);
  }
  return texCube(p, 1, wp, 0.f);
}

// IBLIrradianceSoft.h:75-101: cosine-weighted hemisphere sum, sampleDelta 0.025
__device__ inline float4 fsIrradiance(const DrawParams &p, const FragIn &f) {
  const float PI = 3.14159265359f;
  f3 N = normalize3(f.v.v3(0));
  f3 irradiance = mk3(0.f, 0.f, 0.f);
  f3 up = mk3(0.0f, 1.0f, 0.0f);
  f3 right = normalize3(cross3(up, N));
  up = normalize3(cross3(N, right));
  const float sampleDelta = 0.025f;
  float nrSamples = 0.0f;
  for (float phi = 0.0f; phi < 2.0f * PI; phi += sampleDelta) {
    float sp = sinf(phi), cp = cosf(phi);
    for (float theta = 0.0f; theta < 0.5f * PI; theta += sampleDelta) {
      float st = sinf(theta), ct = cosf(theta);
      f3 ts = mk3(st * cp, st * sp, ct);
      f3 sampleVec = right * ts.x + up * ts.y + N * ts.z;
      float4 c = texCube(p, 0, sampleVec, 0.f);
      irradiance = irradiance + mk3(c.x, c.y, c.z) * ct * st;
      nrSamples++;
    }
  }
  irradiance = PI * irradiance * (1.0f / nrSamples);
  return make_float4(irradiance.x, irradiance.y, irradiance.z, 1.0f);
}

// IBLPrefilterSoft.h:101-170: GGX importance sampling, 1024 Hammersley samples, PDF-based source LOD
__device__ __forceinline__ float radicalInverseVdC(uint32_t bits) {
  bits = (bits << 16u) | (bits >> 16u);
  bits = ((bits & 0x55555555u) << 1u) | ((bits & 0xAAAAAAAAu) >> 1u);
  bits = ((bits & 0x33333333u) << 2u) | ((bits & 0xCCCCCCCCu) >> 2u);
  bits = ((bits & 0x0F0F0F0Fu) << 4u) | ((bits & 0xF0F0F0F0u) >> 4u);
  bits = ((bits & 0x00FF00FFu) << 8u) | ((bits & 0xFF00FF00u) >> 8u);
  return (float) ((double) bits * 2.3283064365386963e-10);
}

__device__ inline float4 fsPrefilter(const DrawParams &p, const FragIn &f) {
  const float PI = 3.14159265359f;
  const float srcResolution = uF32(f.U, 256), roughness = uF32(f.U, 260);
  f3 N = normalize3(f.v.v3(0));
  f3 V = N;
  const uint32_t SAMPLE_COUNT = 1024u;
  f3 color = mk3(0.f, 0.f, 0.f);
  float totalWeight = 0.0f;
  const float a = roughness * roughness;
  f3 upv = fabsf(N.z) < 0.999 ? mk3(0.0f, 0.0f, 1.0f) : mk3(1.0f, 0.0f, 0.0f);
  f3 tangent = normalize3(cross3(upv, N));
  f3 bitangent = cross3(N, tangent);
  for (uint32_t i = 0u; i < SAMPLE_COUNT; ++i) {
    float xi0 = (float) i / (float) SAMPLE_COUNT, xi1 = radicalInverseVdC(i);
    float phi = 2.0f * PI * xi0;
    float cosTheta = sqrtf((1.0f - xi1) / (1.0f + (a * a - 1.0f) * xi1));
    float sinTheta = sqrtf(1.0f - cosTheta * cosTheta);
    f3 H = mk3(cosf(phi) * sinTheta, sinf(phi) * sinTheta, cosTheta);
    H = normalize3(tangent * H.x + bitangent * H.y + N * H.z);
    f3 L = normalize3(2.0f * dot3(V, H) * H - V);
    float NdotL = gmax(dot3(N, L), 0.0f);
    if (NdotL > 0.0f) {
      float a2 = a * a;
      float NdotH = gmax(dot3(N, H), 0.0f);
      float NdotH2 = NdotH * NdotH;
      float denom = (NdotH2 * (a2 - 1.0f) + 1.0f);
      denom = PI * denom * denom;
      float D = a2 / denom;
      float NdotHb = gmax(dot3(N, H), 0.0f);
      float HdotV = gmax(dot3(H, V), 0.0f);
      float pdf = D * NdotHb / (4.0f * HdotV) + 0.0001f;
      float saTexel = 4.0f * PI / (6.0f * srcResolution * srcResolution);
      float saSample = 1.0f / ((float) SAMPLE_COUNT * pdf + 0.0001f);
      float mipLevel = roughness == 0.0f ? 0.0f : 0.5f * log2f(saSample / saTexel);
      float4 c = texCube(p, 0, L, mipLevel);
      color = color + mk3(c.x, c.y, c.z) * NdotL;
      totalWeight += NdotL;
    }
  }
  color = color / totalWeight;
  return make_float4(color.x, color.y, color.z, 1.0f);
}

// ---- FXAA post pass (QuadFilter + FxaaSoft.h) ------------------------------------------------------
// QUALITY(q) of FxaaSoft.h:74
__device__ __forceinline__ float fxaaQuality(float q) {
  return q < 5.f ? 1.0f : (q > 5.f ? (q < 10.f ? 2.0f : (q < 11.f ? 4.0f : 8.0f)) : 1.5f);
}
__device__ __forceinline__ float rgb2luma(f3 c) { return dot3(c, mk3(0.299f, 0.587f, 0.114f)); }
__device__ __forceinline__ float fxaaClamp01(float x) { return gclamp(x, 0.0f, 1.0f); }
__device__ __forceinline__ f3 fxaaTex(const DrawParams &p, float u, float v) {
  const float4 c = textureRGBA8(p.samp[0], 0, u, v, 0.f);
  return mk3(div255(c.x), div255(c.y), div255(c.z));
}
__device__ __forceinline__ f3 fxaaTexOff(const DrawParams &p, float u, float v, int ox, int oy) {
  float4 c = unpackUnit4(textureOffsetImpl(p.samp[0], u, v, ox, oy));
  return mk3(c.x, c.y, c.z);
}

__device__ inline f3 fxaaColor(const DrawParams &p, const FragIn &f) {
  // FxaaSoft.h:83-262 (FXAA 3.11-style edge walk: 12 iterations, subpixel quality 0.75)
  const float inv_x = 1.0f / uF32(f.U, 0), inv_y = 1.0f / uF32(f.U, 4);
  const float tu = f.v[0], tv = f.v[1];
  f3 colorCenter = fxaaTex(p, tu, tv);
  float lumaCenter = rgb2luma(colorCenter);
  float lumaDown = rgb2luma(fxaaTexOff(p, tu, tv, 0, -1));
  float lumaUp = rgb2luma(fxaaTexOff(p, tu, tv, 0, 1));
  float lumaLeft = rgb2luma(fxaaTexOff(p, tu, tv, -1, 0));
  float lumaRight = rgb2luma(fxaaTexOff(p, tu, tv, 1, 0));
  float lumaMin = gmin(lumaCenter, gmin(gmin(lumaDown, lumaUp), gmin(lumaLeft, lumaRight)));
  float lumaMax = gmax(lumaCenter, gmax(gmax(lumaDown, lumaUp), gmax(lumaLeft, lumaRight)));
  float lumaRange = lumaMax - lumaMin;
  if (lumaRange < gmax(0.0312f, lumaMax * 0.125f)) return colorCenter;
  float lumaDownLeft = rgb2luma(fxaaTexOff(p, tu, tv, -1, -1));
  float lumaUpRight = rgb2luma(fxaaTexOff(p, tu, tv, 1, 1));
  float lumaUpLeft = rgb2luma(fxaaTexOff(p, tu, tv, -1, 1));
  float lumaDownRight = rgb2luma(fxaaTexOff(p, tu, tv, 1, -1));
  float lumaDownUp = lumaDown + lumaUp;
  float lumaLeftRight = lumaLeft + lumaRight;
  float lumaLeftCorners = lumaDownLeft + lumaUpLeft;
  float lumaDownCorners = lumaDownLeft + lumaDownRight;
  float lumaRightCorners = lumaDownRight + lumaUpRight;
  float lumaUpCorners = lumaUpRight + lumaUpLeft;
  float edgeHorizontal = fabsf(-2.0f * lumaLeft + lumaLeftCorners) + fabsf(-2.0f * lumaCenter + lumaDownUp) * 2.0f +
                         fabsf(-2.0f * lumaRight + lumaRightCorners);
  float edgeVertical = fabsf(-2.0f * lumaUp + lumaUpCorners) + fabsf(-2.0f * lumaCenter + lumaLeftRight) * 2.0f +
                       fabsf(-2.0f * lumaDown + lumaDownCorners);
  bool isHorizontal = (edgeHorizontal >= edgeVertical);
  float stepLength = isHorizontal ? inv_y : inv_x;
  float luma1 = isHorizontal ? lumaDown : lumaLeft;
  float luma2 = isHorizontal ? lumaUp : lumaRight;
  float gradient1 = luma1 - lumaCenter;
  float gradient2 = luma2 - lumaCenter;
  bool is1Steepest = fabsf(gradient1) >= fabsf(gradient2);
  float gradientScaled = 0.25f * gmax(fabsf(gradient1), fabsf(gradient2));
  float lumaLocalAverage = 0.0f;
  if (is1Steepest) {
    stepLength = -stepLength;
    lumaLocalAverage = 0.5f * (luma1 + lumaCenter);
  } else {
    lumaLocalAverage = 0.5f * (luma2 + lumaCenter);
  }
  float cu = tu, cv = tv;
  if (isHorizontal) cv += stepLength * 0.5f;
  else cu += stepLength * 0.5f;
  float offx = isHorizontal ? inv_x : 0.0f, offy = isHorizontal ? 0.0f : inv_y;
  float u1 = cu - offx * fxaaQuality(0.f), v1 = cv - offy * fxaaQuality(0.f);
  float u2 = cu + offx * fxaaQuality(0.f), v2 = cv + offy * fxaaQuality(0.f);
  float lumaEnd1 = 0.f, lumaEnd2 = 0.f;
  bool reached1 = false, reached2 = false, reachedBoth = false;
  for (int i = 1; i < 12; i++) {
    if (!reached1) {
      lumaEnd1 = rgb2luma(fxaaTex(p, u1, v1));
      lumaEnd1 = lumaEnd1 - lumaLocalAverage;
      reached1 = fabsf(lumaEnd1) >= gradientScaled;
    }
    if (!reached2) {
      lumaEnd2 = rgb2luma(fxaaTex(p, u2, v2));
      lumaEnd2 = lumaEnd2 - lumaLocalAverage;
      reached2 = fabsf(lumaEnd2) >= gradientScaled;
    }
    reachedBoth = reached1 && reached2;
    if (!reached1) {
      u1 -= offx * fxaaQuality((float) i);
      v1 -= offy * fxaaQuality((float) i);
    }
    if (!reached2) {
      u2 += offx * fxaaQuality((float) i);
      v2 += offy * fxaaQuality((float) i);
    }
    if (reachedBoth) break;
  }
  float distance1 = isHorizontal ? (tu - u1) : (tv - v1);
  float distance2 = isHorizontal ? (u2 - tu) : (v2 - tv);
  bool isDirection1 = distance1 < distance2;
  float distanceFinal = gmin(distance1, distance2);
  bool isLumaCenterSmaller = lumaCenter < lumaLocalAverage;
  bool correctVariation1 = (lumaEnd1 < 0.0f) != isLumaCenterSmaller;
  bool correctVariation2 = (lumaEnd2 < 0.0f) != isLumaCenterSmaller;
  bool correctVariation = isDirection1 ? correctVariation1 : correctVariation2;
  float edgeLength = (distance1 + distance2);
  float pixelOffset = -distanceFinal / edgeLength + 0.5f;
  float finalOffset = correctVariation ? pixelOffset : 0.0f;
  float lumaAverage = (1.0f / 12.0f) * (2.0f * (lumaDownUp + lumaLeftRight) + lumaLeftCorners + lumaRightCorners);
  float subPixelOffset1 = fxaaClamp01(fabsf(lumaAverage - lumaCenter) / lumaRange);
  float subPixelOffset2 = (-2.0f * subPixelOffset1 + 3.0f) * subPixelOffset1 * subPixelOffset1;
  float subPixelOffsetFinal = subPixelOffset2 * subPixelOffset2 * 0.75f;
  finalOffset = gmax(finalOffset, subPixelOffsetFinal);
  float fu = tu, fv = tv;
  if (isHorizontal) fv += finalOffset * stepLength;
  else fu += finalOffset * stepLength;
  return fxaaTex(p, fu, fv);
}

template<int SH>
__device__ __forceinline__ float4 runFS(const DrawParams &p, const FragIn &f) {
  if (SH == SH_BASE) return uV4(f.U, 256 + 32);
  if (SH == SH_SKYBOX) return fsSkybox(p, f);
  if (SH == SH_IBL_IRR) return fsIrradiance(p, f);
  if (SH == SH_IBL_PRE) return fsPrefilter(p, f);
  if (SH == SH_FXAA) {
    f3 c = fxaaColor(p, f);
    return make_float4(c.x, c.y, c.z, 1.f);
  }
  if (SH == SH_VCOLOR) return make_float4(f.v[0], f.v[1], f.v[2], f.v[3]);
  if (SH == SH_BLINN) return fsBlinnPhong<false>(p, f);
  if (SH == SH_BLINN_DIR) return fsBlinnPhong<true>(p, f);
  return fsPbr<SH == SH_PBR_CAPTURE>(p, f);
}

// does the FS read texcoord derivatives (any bound 2D sampler with a mip filter and LOD callback)
__device__ __forceinline__ bool needsDerivatives(const DrawParams &p) {
  for (int s = 0; s < 4; s++)
    if (p.samp[s].valid && p.samp[s].lodFromDerivative && p.def[s]) return true;
  return false;
}

}  // namespace sglc
