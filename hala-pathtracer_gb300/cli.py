#!/usr/bin/env python3
"""Headless renderer CLI, the counterpart of src/bin/hala-pathtracer.rs.

    python hala-pathtracer_gb300/cli.py --workload disney_grid_1080p_64spp [--frames N] [--out PREFIX]
    python hala-pathtracer_gb300/cli.py -c conf/config.yaml [--frames N] [--out PREFIX]

`--workload` renders one of the procedural scenes; `-c` reads the reference's
YAML schema (window, tracer, scene_file, hdri_*, colours). The window and
interactive "Save" button of the reference become `--out`, which writes
<PREFIX>_color.pfm, _albedo.pfm, _normal.pfm, _final.ppm and _final.png.
"""
import argparse
import importlib
import os
import sys
import time

# the texture the reference loads before its scene (src/bin/hala-pathtracer.rs:195)
BLUE_NOISE = "./assets/textures/blue_noise.png"

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def resolve(path, config_dir):
    """A config path: as given (relative to the working directory, like the
    reference binary run from its checkout), else next to the config file or
    its parent directory."""
    if os.path.isabs(path) or os.path.exists(path):
        return path
    for base in (config_dir, os.path.dirname(config_dir)):
        p = os.path.join(base, path)
        if os.path.exists(p):
            return p
    return path


def main(argv=None):
    pt = importlib.import_module("hala-pathtracer_gb300")
    scenes = importlib.import_module("hala-pathtracer_gb300.scenes")
    ap = argparse.ArgumentParser(description="GB300 wavefront path tracer")
    ap.add_argument("-c", "--config", help="conf/*.yaml file (reference schema)")
    ap.add_argument("--workload", help="procedural workload: " + ", ".join(sorted(scenes.WORKLOADS)))
    ap.add_argument("--frames", type=int, default=0, help="frames (1 spp each); default: the workload's spp")
    ap.add_argument("--out", default="", help="image prefix for save_images")
    ap.add_argument("--seed", type=int, default=None)
    ap.add_argument("--wave", type=int, default=0, help="paths per wavefront (0 = library default)")
    ap.add_argument("--blue-noise", default=None,
                    help=f"camera-jitter texture (default with -c: {BLUE_NOISE} where it exists, "
                         "else the built-in substitute)")
    args = ap.parse_args(argv)
    if bool(args.config) == bool(args.workload):
        ap.error("give exactly one of -c/--config or --workload")
    if args.config:
        cfgmod = importlib.import_module("hala-pathtracer_gb300.config")
        cfg = cfgmod.load_app_config(args.config)
        cfgmod.validate_app_config(cfg, check_scene_file=False)
        loader = importlib.import_module("hala-pathtracer_gb300.gltf")
        base = os.path.dirname(os.path.abspath(args.config))
        scene_path = resolve(cfg.scene_file, base)
        if not os.path.exists(scene_path):
            raise cfgmod.ConfigError(f'The scene file "{cfg.scene_file}" is not found.')
        scene = loader.load_scene(scene_path, cfg.window.width, cfg.window.height)
        env = cfgmod.environment_settings(cfg)
        r = pt.Renderer(cfgmod.tracer_config(cfg, seed=args.seed or 0, wave_paths=args.wave))
        bn = resolve(args.blue_noise or BLUE_NOISE, base)
        if args.blue_noise or os.path.exists(bn):
            r.load_blue_noise_texture(bn)
        r.set_scene(scene)
        if env["hdri_file"]:
            exr = importlib.import_module("hala-pathtracer_gb300.exr")
            r.set_envmap(exr.read_rgb(resolve(env["hdri_file"], base)), env["hdri_rotation"])
        else:
            r.set_ground_color(env["ground_color"])
            r.set_sky_color(env["sky_color"])
        r.set_env_intensity(env["env_intensity"])
        r.set_exposure_value(env["exposure_value"])
        r.commit()
        frames = args.frames or max(1, cfg.tracer.max_samples or 1)
    else:
        fn = scenes.WORKLOADS[args.workload]
        scene = fn()
        if args.seed is not None:
            scene.seed = args.seed
        r = pt.renderer_for(scene, wave_paths=args.wave)
        frames = args.frames or scene.spp
    t0 = time.perf_counter()
    r.render(frames)
    r.wait_idle()
    dt = time.perf_counter() - t0
    st = r.stats()
    print(f"rendered {st.paths} paths in {st.render_ms:.2f} ms device / {dt * 1e3:.2f} ms wall: "
          f"{st.paths / max(st.render_ms, 1e-9) / 1e3:.2f} Mpaths/s, "
          f"{(st.closest_rays + st.shadow_rays) / max(st.render_ms, 1e-9) / 1e6:.3f} Grays/s, "
          f"BVH build {st.bvh_build_ms:.2f} ms", flush=True)
    if args.out:
        r.save_images(args.out)
        png = importlib.import_module("hala-pathtracer_gb300.png")
        png.write(args.out + "_final.png", r.image(pt.abi.IMAGE_FINAL)[..., :3])
        print(f"wrote {args.out}_color.pfm, _albedo.pfm, _normal.pfm, _final.ppm, _final.png")
    r.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
