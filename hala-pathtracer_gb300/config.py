"""The conf/*.yaml schema of the reference (src/config/{mod,tracer,window}.rs).

    window:  {width, height}
    tracer:  {max_depth, rr_depth, exposure_value,
              tonemap: {enable, enable_aces, use_simple_aces}, max_samples}
    scene_file, hdri_file, hdri_rotation, ground_color, sky_color, env_intensity

Parsing uses a small YAML-subset reader (block mappings, scalars, flow
lists, comments), enough for every file under conf/ of the reference; no
YAML library is required. Defaults and validation follow the Rust serde
structs line by line.
"""
import dataclasses
import os

from . import abi


class ConfigError(ValueError):
    pass


def _scalar(tok):
    t = tok.strip()
    if t == "" or t in ("~", "null", "Null", "NULL"):
        return None
    if t in ("true", "True", "TRUE"):
        return True
    if t in ("false", "False", "FALSE"):
        return False
    if t.startswith("[") and t.endswith("]"):
        inner = t[1:-1].strip()
        return [] if not inner else [_scalar(x) for x in inner.split(",")]
    if (t[0] == t[-1]) and t[0] in "'\"" and len(t) >= 2:
        return t[1:-1]
    try:
        return int(t, 0) if t.lstrip("+-").isdigit() else float(t)
    except ValueError:
        return t


def parse_yaml(text):
    """Parses the YAML subset of conf/*.yaml into nested dicts."""
    root = {}
    stack = [(-1, root)]
    for lineno, raw in enumerate(text.splitlines(), 1):
        line = raw.split(" #")[0].rstrip() if not raw.lstrip().startswith("#") else ""
        if not line.strip():
            continue
        indent = len(line) - len(line.lstrip(" "))
        body = line.strip()
        if ":" not in body:
            raise ConfigError(f"line {lineno}: expected 'key: value'")
        key, _, val = body.partition(":")
        key = key.strip()
        while stack and indent <= stack[-1][0]:
            stack.pop()
        if not stack:
            raise ConfigError(f"line {lineno}: bad indentation")
        parent = stack[-1][1]
        if val.strip() == "":
            child = {}
            parent[key] = child
            stack.append((indent, child))
        else:
            parent[key] = _scalar(val)
    return root


@dataclasses.dataclass
class TonemapConfig:  # src/config/tracer.rs:5-13
    enable: bool = False
    enable_aces: bool = False
    use_simple_aces: bool = False


@dataclasses.dataclass
class TracerConfig:  # src/config/tracer.rs:15-39
    max_depth: int = 1
    rr_depth: int = 0
    exposure_value: float = 0.0
    tonemap: TonemapConfig = dataclasses.field(default_factory=TonemapConfig)
    max_samples: int = 0


@dataclasses.dataclass
class WindowConfig:  # src/config/window.rs:5-9
    width: int = 0
    height: int = 0


@dataclasses.dataclass
class AppConfig:  # src/config/mod.rs:22-36
    window: WindowConfig
    tracer: TracerConfig
    scene_file: str
    hdri_file: str = ""
    hdri_rotation: float = 0.0
    ground_color: tuple = (0.5, 0.5, 0.5)
    sky_color: tuple = (0.5, 0.5, 0.5)
    env_intensity: float = 1.0


def app_config_from_dict(d):
    if "window" not in d or "tracer" not in d or "scene_file" not in d:
        raise ConfigError("missing field: window, tracer and scene_file are required")
    w = d["window"] or {}
    t = d["tracer"] or {}
    tm = t.get("tonemap") or {}
    if "width" not in w or "height" not in w:
        raise ConfigError("missing field: window.width/height")

    def u16(v, name):
        if v is None:
            return 0
        if not isinstance(v, int) or isinstance(v, bool) or not (0 <= v <= 65535):
            raise ConfigError(f"{name} must be an integer in [0, 65535]")
        return v

    hdri = d.get("hdri_file")
    return AppConfig(
        window=WindowConfig(u16(w.get("width"), "window.width"), u16(w.get("height"), "window.height")),
        tracer=TracerConfig(
            max_depth=u16(t.get("max_depth", 0), "tracer.max_depth"),
            rr_depth=u16(t.get("rr_depth", 0), "tracer.rr_depth"),
            exposure_value=float(t.get("exposure_value") or 0.0),
            tonemap=TonemapConfig(bool(tm.get("enable", False)), bool(tm.get("enable_aces", False)),
                                  bool(tm.get("use_simple_aces", False))),
            max_samples=int(t.get("max_samples") or 0)),
        scene_file=str(d["scene_file"]),
        hdri_file="" if hdri is None else str(hdri),
        hdri_rotation=float(d.get("hdri_rotation") or 0.0),
        ground_color=tuple(float(x) for x in (d.get("ground_color") or (0.5, 0.5, 0.5))),
        sky_color=tuple(float(x) for x in (d.get("sky_color") or (0.5, 0.5, 0.5))),
        env_intensity=float(d["env_intensity"]) if d.get("env_intensity") is not None else 1.0,
    )


def load_app_config(path):
    """src/config/mod.rs:53-58"""
    try:
        with open(path) as f:
            text = f.read()
    except OSError as e:
        raise ConfigError(f"Failed to read the config file: {path}") from e
    try:
        return app_config_from_dict(parse_yaml(text))
    except ConfigError as e:
        raise ConfigError(f"Failed to parse the config file: {path}: {e}") from e


def validate_app_config(cfg, check_scene_file=True, base_dir=None):
    """src/config/mod.rs:41-50, window.rs:13-21, tracer.rs:43-49"""
    if cfg.window.width == 0:
        raise ConfigError("The width is 0.")
    if cfg.window.height == 0:
        raise ConfigError("The height is 0.")
    if cfg.tracer.rr_depth > cfg.tracer.max_depth:
        raise ConfigError("The Russian Roulette depth is greater than the max depth.")
    if check_scene_file:
        p = cfg.scene_file if base_dir is None else os.path.join(base_dir, cfg.scene_file)
        if not os.path.exists(p):
            raise ConfigError(f'The scene file "{cfg.scene_file}" is not found.')


def tracer_config(cfg, seed=0, wave_paths=0, keep_samples=False):
    """The HalaRenderer::new arguments of src/bin/hala-pathtracer.rs:128-138."""
    return abi.make_config(cfg.window.width, cfg.window.height, cfg.tracer.max_depth, cfg.tracer.rr_depth,
                           cfg.tracer.tonemap.enable, cfg.tracer.tonemap.enable_aces,
                           cfg.tracer.tonemap.use_simple_aces, seed=seed,
                           max_samples=cfg.tracer.max_samples, wave_paths=wave_paths, keep_samples=keep_samples)


def environment_settings(cfg):
    """What src/bin/hala-pathtracer.rs:201-208 passes to the renderer: the
    sky colour is multiplied by 4 there before set_sky_color."""
    return {
        "hdri_file": cfg.hdri_file,
        "hdri_rotation": cfg.hdri_rotation,
        "ground_color": tuple(cfg.ground_color) + (1.0,),
        "sky_color": tuple(c * 4.0 for c in cfg.sky_color) + (1.0,),
        "env_intensity": cfg.env_intensity,
        "exposure_value": cfg.tracer.exposure_value,
    }
