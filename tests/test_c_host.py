"""The C ABI from a plain C host: a C99 program that includes
include/hala_pt.h (compiled with -std=c99 -pedantic -Werror) and links
libhalapt.so reads a glTF scene and an OpenEXR environment through the
library's own readers and prints what it got; the numbers equal those of the
Python loaders of the same files (on the CPU: that program makes no CUDA
call). On a GPU, a second C program drives a whole render through the C ABI
alone and gets the Python host's images bit for bit. This is the path a
non-Python host (the reference's Rust binary over an FFI crate, a cgo or JNI
binding) takes."""
import importlib
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

C_HOST = r"""
#include <stdio.h>
#include <stdlib.h>
#include "hala_pt.h"

int main(int argc, char** argv) {
  char err[256];
  pt_gltf_scene* scene = NULL;
  pt_status st;
  const pt_scene_desc* d;
  unsigned long long nv = 0, ni = 0, ntex = 0;
  double vsum = 0.0, tsum = 0.0, esum = 0.0;
  uint32_t i, w = 0, h = 0;
  size_t k;
  float* rgb;
  if (argc != 3) return 2;
  st = pt_gltf_load(argv[1], &scene, err, sizeof err);
  if (st != PT_OK) {
    printf("gltf error %d %s\n", (int)st, err);
    return 1;
  }
  d = pt_gltf_scene_desc(scene);
  for (i = 0; i < d->num_primitives; ++i) {
    const pt_primitive* p = &d->primitives[i];
    nv += p->num_vertices;
    ni += p->num_indices;
    for (k = 0; k < 11u * p->num_vertices; ++k) vsum += p->vertices[k];
  }
  for (i = 0; i < d->num_textures; ++i) {
    const pt_texture* t = &d->textures[i];
    ntex += (unsigned long long)t->width * t->height;
    for (k = 0; k < 4u * t->width * t->height; ++k) tsum += t->rgba[k];
  }
  printf("scene %u %u %u %u %u %llu %llu %llu %u %.9g %.9g\n", d->num_primitives, d->num_materials,
         d->num_lights, d->num_cameras, d->num_textures, nv, ni, ntex, pt_gltf_skipped_images(scene), vsum, tsum);
  pt_gltf_free(scene);
  st = pt_exr_read_rgb(argv[2], NULL, 0, &w, &h, err, sizeof err);
  if (st != PT_OK) {
    printf("exr error %d %s\n", (int)st, err);
    return 1;
  }
  rgb = (float*)malloc(sizeof(float) * 3u * w * h);
  if (!rgb) return 3;
  st = pt_exr_read_rgb(argv[2], rgb, 3u * (size_t)w * h, &w, &h, err, sizeof err);
  if (st != PT_OK) {
    printf("exr error %d %s\n", (int)st, err);
    return 1;
  }
  for (k = 0; k < 3u * (size_t)w * h; ++k) esum += rgb[k];
  printf("exr %u %u %.9g\n", w, h, esum);
  free(rgb);
  return 0;
}
"""


def test_c99_host_reads_scene_and_environment(pt, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pt.build()
    from tests.test_gltf_c import _document
    import base64
    import json
    gltf = importlib.import_module("hala-pathtracer_gb300.gltf")
    exr = importlib.import_module("hala-pathtracer_gb300.exr")
    doc, blob = _document(tmp_path)
    doc = dict(doc, buffers=[{"byteLength": len(blob), "uri": "data:application/octet-stream;base64," +
                              base64.b64encode(blob).decode()}])
    scene_path = tmp_path / "scene.gltf"
    scene_path.write_text(json.dumps(doc))
    env = np.random.default_rng(5).random((16, 32, 3)).astype(np.float32) * 4.0
    env_path = str(tmp_path / "sky.exr")
    exr.write(env_path, env, half=False, compression="ZIP")

    src = tmp_path / "host.c"
    src.write_text(C_HOST)
    build = os.path.join(ROOT, "hala-pathtracer_gb300", "_build")
    exe = str(tmp_path / "host")
    r = subprocess.run([cc, "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                        str(src), "-L", build, "-lhalapt", "-Wl,-rpath," + build, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, str(scene_path), env_path], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = dict((ln.split()[0], ln.split()[1:]) for ln in r.stdout.splitlines())

    s = gltf.load_scene(str(scene_path))
    nv = sum(len(v) for v, _, _, _ in s.meshes)
    ni = sum(len(i) for _, i, _, _ in s.meshes)
    ntex = sum(t.shape[0] * t.shape[1] for t in s.textures)
    got = lines["scene"]
    assert [int(x) for x in got[:9]] == [len(s.meshes), len(s.materials), len(s.lights), len(s.cameras),
                                          len(s.textures), nv, ni, ntex, len(s.skipped_images)]
    vsum = sum(float(np.sum(v.astype(np.float64))) for v, _, _, _ in s.meshes)
    tsum = sum(float(np.sum(t.astype(np.float64))) for t in s.textures)
    assert float(got[9]) == pytest.approx(vsum, rel=1e-7, abs=1e-9)
    assert float(got[10]) == pytest.approx(tsum, rel=1e-6)
    w, h, esum = lines["exr"]
    assert (int(w), int(h)) == (32, 16)
    assert float(esum) == pytest.approx(float(np.sum(exr.read_rgb(env_path).astype(np.float64))), rel=1e-7)


C_RENDER = r"""
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "hala_pt.h"

/* hala-pathtracer's before_run + render loop from C: create, blue-noise
   texture, scene file, environment colours, commit, render, read back. */
int main(int argc, char** argv) {
  pt_tracer_config cfg;
  pt_renderer* r = NULL;
  const float ground[4] = {0.1f, 0.1f, 0.1f, 1.0f}, sky[4] = {0.8f, 0.9f, 1.6f, 1.0f};
  float* accum;
  unsigned char* final_img;
  FILE* f;
  pt_status st;
  if (argc != 5) return 2;
  memset(&cfg, 0, sizeof cfg);
  cfg.width = 48;
  cfg.height = 32;
  cfg.max_depth = 6;
  cfg.rr_depth = 3;
  cfg.enable_tonemap = 1;
  cfg.enable_aces = 1;
  cfg.wave_paths = 1u << 16;
  st = pt_renderer_create(&cfg, &r);
  if (st != PT_OK) return 10 + (int)st;
  if ((st = pt_renderer_load_blue_noise_texture(r, argv[2])) != PT_OK ||
      (st = pt_renderer_set_scene_file(r, argv[1])) != PT_OK ||
      (st = pt_renderer_set_ground_color(r, ground)) != PT_OK || (st = pt_renderer_set_sky_color(r, sky)) != PT_OK ||
      (st = pt_renderer_set_exposure_value(r, 0.5f)) != PT_OK || (st = pt_renderer_commit(r)) != PT_OK ||
      (st = pt_renderer_render(r, 3)) != PT_OK) {
    printf("error %d: %s\n", (int)st, pt_renderer_last_error(r));
    pt_renderer_destroy(r);
    return 1;
  }
  accum = (float*)malloc(sizeof(float) * 4u * 48u * 32u);
  final_img = (unsigned char*)malloc(4u * 48u * 32u);
  if (!accum || !final_img) return 3;
  if (pt_renderer_read_image(r, PT_IMAGE_ACCUM, accum, sizeof(float) * 4u * 48u * 32u) != PT_OK ||
      pt_renderer_read_image(r, PT_IMAGE_FINAL, final_img, 4u * 48u * 32u) != PT_OK) {
    printf("error: %s\n", pt_renderer_last_error(r));
    return 1;
  }
  f = fopen(argv[3], "wb");
  if (!f) return 4;
  fwrite(accum, sizeof(float), 4u * 48u * 32u, f);
  fclose(f);
  f = fopen(argv[4], "wb");
  if (!f) return 4;
  fwrite(final_img, 1, 4u * 48u * 32u, f);
  fclose(f);
  free(accum);
  free(final_img);
  pt_renderer_destroy(r);
  return 0;
}
"""


@pytest.mark.gpu
def test_c99_host_renders_like_the_python_host(pt, tmp_path):
    """A C program drives a whole render through the C ABI alone (blue-noise
    texture and scene read from files by the library) and gets the images
    of the Python host's render of the same files, bit for bit."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pt.build()
    import base64
    import json
    from tests.test_gltf_c import _document, _png
    gltf = importlib.import_module("hala-pathtracer_gb300.gltf")
    abi = importlib.import_module("hala-pathtracer_gb300.abi")
    doc, blob = _document(tmp_path)
    doc = dict(doc, buffers=[{"byteLength": len(blob), "uri": "data:application/octet-stream;base64," +
                              base64.b64encode(blob).decode()}])
    scene_path = tmp_path / "scene.gltf"
    scene_path.write_text(json.dumps(doc))
    tex = np.random.default_rng(21).integers(0, 256, (1024, 1024, 4)).astype(np.uint8)
    bn_path = tmp_path / "blue_noise.png"
    bn_path.write_bytes(_png(tex, 8, 6))
    src = tmp_path / "render.c"
    src.write_text(C_RENDER)
    build = os.path.join(ROOT, "hala-pathtracer_gb300", "_build")
    exe = str(tmp_path / "render")
    r = subprocess.run([cc, "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                        str(src), "-L", build, "-lhalapt", "-Wl,-rpath," + build, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    acc_path, fin_path = tmp_path / "accum.f32", tmp_path / "final.u8"
    r = subprocess.run([exe, str(scene_path), str(bn_path), str(acc_path), str(fin_path)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr

    s = gltf.load_scene(str(scene_path), 48, 32)
    s.max_depth, s.rr_depth = 6, 3
    s.tonemap = (True, True, False)
    s.ground_color, s.sky_color, s.exposure_value = (0.1, 0.1, 0.1, 1.0), (0.8, 0.9, 1.6, 1.0), 0.5
    s.blue_noise = tex
    h = pt.renderer_for(s, wave_paths=1 << 16)
    h.render(3)
    acc = np.fromfile(acc_path, np.float32).reshape(32, 48, 4)
    fin = np.fromfile(fin_path, np.uint8).reshape(32, 48, 4)
    assert np.array_equal(acc.view(np.uint32), h.image(abi.IMAGE_ACCUM).view(np.uint32))
    assert np.array_equal(fin, h.image(abi.IMAGE_FINAL))
    h.close()
