// Test infrastructure: a recording implementation of the C ABI of include/softgl_cuda.h (the calls
// the C++ binding softglrender_gb300/host/RendererCUDA.cpp makes, and the multi-scene extension a
// C++ caller makes with the binding's handles). Linked in place of the CUDA library, it performs
// nothing: every call is written as one text line to the file named by SGLC_TRACE,
// "<function> <argument>...", each argument tagged
//   i:<int>  an integer        h:<n> a handle created earlier in the trace
//   o:<n>    a handle created by this call        s:<hex> a string        b:<hex> bytes
//   H:<n>,<n>,...  an array of handles created earlier
// Structures travel as their bytes (the same layout on every little-endian host the tests use).
// tests/trace_replay.py replays such a trace through any library that exports the ABI (the CUDA
// renderer, the CPU oracle, the reference-backed checker) and returns the images read back.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "softgl_cuda.h"

namespace {

FILE *g_out = nullptr;
int g_next = 1;
char g_ctx;   // the one context's address

FILE *out() {
  if (!g_out) {
    const char *path = getenv("SGLC_TRACE");
    g_out = fopen(path ? path : "sglc_trace.txt", "w");
  }
  return g_out;
}

void hex(const void *p, size_t n) {
  const unsigned char *b = static_cast<const unsigned char *>(p);
  for (size_t i = 0; i < n; i++) fprintf(out(), "%02x", b[i]);
}

void beginCall(const char *name) { fprintf(out(), "%s", name); }
void argI(long long v) { fprintf(out(), " i:%lld", v); }
void argH(sglc_handle h) { fprintf(out(), " h:%d", (int) h); }
void argS(const char *s) {
  fprintf(out(), " s:");
  hex(s, strlen(s));
}
void argHs(const sglc_handle *h, int n) {
  fprintf(out(), " H:");
  for (int k = 0; k < n; k++) fprintf(out(), k ? ",%d" : "%d", (int) h[k]);
}
void argB(const void *p, size_t n) {
  fprintf(out(), " b:");
  hex(p, n);
}
sglc_handle argOut(sglc_handle *o) {
  sglc_handle h = g_next++;
  if (o) *o = h;
  fprintf(out(), " o:%d", (int) h);
  return h;
}
sglc_status endCall() {
  fprintf(out(), "\n");
  fflush(g_out);
  return SGLC_OK;
}

}  // namespace

extern "C" {

sglc_status sglc_create(sglc_context **o, int32_t device) {
  beginCall("create");
  argI(device);
  *o = reinterpret_cast<sglc_context *>(&g_ctx);
  return endCall();
}
sglc_status sglc_destroy(sglc_context *) {
  beginCall("destroy");
  return endCall();
}
const char *sglc_last_error(sglc_context *) { return ""; }
sglc_status sglc_release(sglc_context *, sglc_handle h) {
  beginCall("release");
  argH(h);
  return endCall();
}
sglc_status sglc_create_framebuffer(sglc_context *, int32_t offscreen, sglc_handle *o) {
  beginCall("create_framebuffer");
  argI(offscreen);
  argOut(o);
  return endCall();
}
sglc_status sglc_framebuffer_set_color_attachment(sglc_context *, sglc_handle fb, sglc_handle tex, int32_t layer,
                                                  int32_t level) {
  beginCall("framebuffer_set_color_attachment");
  argH(fb);
  argH(tex);
  argI(layer);
  argI(level);
  return endCall();
}
sglc_status sglc_framebuffer_set_depth_attachment(sglc_context *, sglc_handle fb, sglc_handle tex) {
  beginCall("framebuffer_set_depth_attachment");
  argH(fb);
  argH(tex);
  return endCall();
}
sglc_status sglc_framebuffer_is_valid(sglc_context *, sglc_handle, int32_t *valid) {
  *valid = 1;
  return SGLC_OK;
}
sglc_status sglc_create_texture(sglc_context *, const sglc_texture_desc *d, sglc_handle *o) {
  beginCall("create_texture");
  argB(d, sizeof(*d));
  argOut(o);
  return endCall();
}
sglc_status sglc_texture_set_sampler_desc(sglc_context *, sglc_handle tex, const sglc_sampler_desc *s) {
  beginCall("texture_set_sampler_desc");
  argH(tex);
  argB(s, sizeof(*s));
  return endCall();
}
sglc_status sglc_texture_init_image_data(sglc_context *, sglc_handle tex) {
  beginCall("texture_init_image_data");
  argH(tex);
  return endCall();
}
sglc_status sglc_texture_set_image_data(sglc_context *, sglc_handle tex, int32_t layer_count,
                                        const void *const *layers, size_t bytes_per_layer) {
  beginCall("texture_set_image_data");
  argH(tex);
  argI(layer_count);
  argI((long long) bytes_per_layer);
  for (int l = 0; l < layer_count; l++) argB(layers[l], bytes_per_layer);
  return endCall();
}
sglc_status sglc_texture_set_level_data(sglc_context *, sglc_handle tex, int32_t layer, int32_t level, const void *data,
                                        size_t bytes) {
  beginCall("texture_set_level_data");
  argH(tex);
  argI(layer);
  argI(level);
  argB(data, bytes);
  return endCall();
}
sglc_status sglc_texture_read_image(sglc_context *, sglc_handle tex, int32_t layer, int32_t level, int32_t resolved,
                                    void *o, size_t bytes) {
  beginCall("texture_read_image");
  argH(tex);
  argI(layer);
  argI(level);
  argI(resolved);
  argI((long long) bytes);
  memset(o, 0, bytes);
  return endCall();
}
sglc_status sglc_texture_store_to_file(sglc_context *, sglc_handle, const char *) { return SGLC_OK; }
sglc_status sglc_texture_load_from_file(sglc_context *, sglc_handle, const char *) { return SGLC_ERR_INVALID_VALUE; }
sglc_status sglc_create_vertex_array(sglc_context *, const void *vertexes, size_t vertexes_len, size_t stride,
                                     const int32_t *indices, size_t indices_len, sglc_handle *o) {
  beginCall("create_vertex_array");
  argB(vertexes, vertexes_len);
  argI((long long) stride);
  argB(indices, indices_len);   // bytes, as VertexArray::indexBufferLength
  argOut(o);
  return endCall();
}
sglc_status sglc_vertex_array_update(sglc_context *, sglc_handle vao, const void *data, size_t len) {
  beginCall("vertex_array_update");
  argH(vao);
  argB(data, len);
  return endCall();
}
sglc_status sglc_create_shader_program(sglc_context *, sglc_handle *o) {
  beginCall("create_shader_program");
  argOut(o);
  return endCall();
}
sglc_status sglc_program_add_define(sglc_context *, sglc_handle prog, const char *name) {
  beginCall("program_add_define");
  argH(prog);
  argS(name);
  return endCall();
}
sglc_status sglc_program_set_shaders(sglc_context *, sglc_handle prog, int32_t model) {
  beginCall("program_set_shaders");
  argH(prog);
  argI(model);
  return endCall();
}
sglc_status sglc_create_pipeline_states(sglc_context *, const sglc_render_states *s, sglc_handle *o) {
  beginCall("create_pipeline_states");
  argB(s, sizeof(*s));
  argOut(o);
  return endCall();
}
sglc_status sglc_create_uniform_block(sglc_context *, const char *name, int32_t size, sglc_handle *o) {
  beginCall("create_uniform_block");
  argS(name);
  argI(size);
  argOut(o);
  return endCall();
}
sglc_status sglc_uniform_block_set_sub_data(sglc_context *, sglc_handle ub, const void *data, int32_t len,
                                            int32_t offset) {
  beginCall("uniform_block_set_sub_data");
  argH(ub);
  argB(data, (size_t) len);
  argI(offset);
  return endCall();
}
sglc_status sglc_uniform_block_set_data(sglc_context *, sglc_handle ub, const void *data, int32_t len) {
  beginCall("uniform_block_set_data");
  argH(ub);
  argB(data, (size_t) len);
  return endCall();
}
sglc_status sglc_create_uniform_sampler(sglc_context *, const char *name, int32_t type, int32_t format,
                                        sglc_handle *o) {
  beginCall("create_uniform_sampler");
  argS(name);
  argI(type);
  argI(format);
  argOut(o);
  return endCall();
}
sglc_status sglc_uniform_sampler_set_texture(sglc_context *, sglc_handle us, sglc_handle tex) {
  beginCall("uniform_sampler_set_texture");
  argH(us);
  argH(tex);
  return endCall();
}
sglc_status sglc_create_shader_resources(sglc_context *, sglc_handle *o) {
  beginCall("create_shader_resources");
  argOut(o);
  return endCall();
}
sglc_status sglc_shader_resources_set_block(sglc_context *, sglc_handle res, int32_t key, sglc_handle ub) {
  beginCall("shader_resources_set_block");
  argH(res);
  argI(key);
  argH(ub);
  return endCall();
}
sglc_status sglc_shader_resources_set_sampler(sglc_context *, sglc_handle res, int32_t key, sglc_handle us) {
  beginCall("shader_resources_set_sampler");
  argH(res);
  argI(key);
  argH(us);
  return endCall();
}
sglc_status sglc_begin_render_pass(sglc_context *, sglc_handle fb, const sglc_clear_states *s) {
  beginCall("begin_render_pass");
  argH(fb);
  argB(s, sizeof(*s));
  return endCall();
}
sglc_status sglc_set_viewport(sglc_context *, int32_t x, int32_t y, int32_t w, int32_t h) {
  beginCall("set_viewport");
  argI(x);
  argI(y);
  argI(w);
  argI(h);
  return endCall();
}
sglc_status sglc_set_vertex_array(sglc_context *, sglc_handle vao) {
  beginCall("set_vertex_array");
  argH(vao);
  return endCall();
}
sglc_status sglc_set_shader_program(sglc_context *, sglc_handle prog) {
  beginCall("set_shader_program");
  argH(prog);
  return endCall();
}
sglc_status sglc_set_shader_resources(sglc_context *, sglc_handle res) {
  beginCall("set_shader_resources");
  argH(res);
  return endCall();
}
sglc_status sglc_set_pipeline_states(sglc_context *, sglc_handle states) {
  beginCall("set_pipeline_states");
  argH(states);
  return endCall();
}
sglc_status sglc_draw(sglc_context *) {
  beginCall("draw");
  return endCall();
}
sglc_status sglc_end_render_pass(sglc_context *) {
  beginCall("end_render_pass");
  return endCall();
}
sglc_status sglc_wait_idle(sglc_context *) {
  beginCall("wait_idle");
  return endCall();
}
sglc_status sglc_set_enable_early_z(sglc_context *, int32_t enable) {
  beginCall("set_enable_early_z");
  argI(enable);
  return endCall();
}
sglc_status sglc_draw_scenes(sglc_context *, const sglc_handle *vaos, const sglc_handle *fbs, const sglc_handle *res,
                             int32_t count, const sglc_clear_states *clear) {
  beginCall("draw_scenes");
  argHs(vaos, count);
  argHs(fbs, count);
  argHs(res, count);
  argI(count);
  argB(clear, sizeof(*clear));
  return endCall();
}

}  // extern "C"
