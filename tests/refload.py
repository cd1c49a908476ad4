"""Loads Pointrix's own Python source (the reference) so that tests execute it
as the checker instead of re-typing its formulas.

TEST INFRASTRUCTURE ONLY.  The files are read from the offline install of the
reference package (``baseline/_ref/pointrix``, made with ``pip install
--no-deps --target baseline/_ref``) or from the directory named by the
environment variable ``PGB_POINTRIX_SRC``; nothing is copied into this
repository.  When neither is present every loader returns ``None`` and the
tests that need live reference code skip; the fixtures that
``tests/golden/make_reference_golden.py`` wrote from the same functions still
run.

Only the configuration and registry machinery around the path is replaced,
because it pulls in packages that are absent on the GPU host (omegaconf,
yaml, tabulate):

* ``pointrix.utils.base.BaseObject`` -- builds ``cfg`` from the class's
  ``Config`` dataclass and calls ``setup`` (the reference parses it through
  omegaconf first, ``pointrix/utils/base.py:28-40``);
* ``pointrix.utils.registry.Registry`` -- ``register()`` returns the class
  unchanged (``pointrix/utils/registry.py:28-45``);
* ``pointrix.utils.config.C`` -- scalar schedules, used by the controller's
  densification decisions only, not by the statistics;
* third-party modules that are absent (``jaxtyping`` for type annotations,
  ``lpips`` which ``loss.py`` imports but ``ssim`` never calls, ``sklearn``'s
  ``NearestNeighbors`` which ``gaussian_utils.py`` imports for the point
  initialiser).

Every function and method the tests call -- ``RenderFeatures``,
``unitquat_to_rotmat``/``quat_to_rotmat``, ``ssim``, the controller's
``preprocess``/``accumulate_viewspace_grad``, ``MsplatRender.render_iter``/
``render_batch`` and ``MsplatNormalRender.render_iter`` -- runs from the
reference file unmodified.
"""
from __future__ import annotations

import contextlib
import importlib.machinery
import importlib.util
import os
import sys
import types
from dataclasses import is_dataclass
from pathlib import Path

REPO = Path(__file__).resolve().parents[1]


def pointrix_dir() -> Path | None:
    """Directory of the reference ``pointrix`` package, or None."""
    cands = []
    env = os.environ.get("PGB_POINTRIX_SRC")
    if env:
        cands += [Path(env), Path(env) / "pointrix"]
    cands.append(REPO / "baseline" / "_ref" / "pointrix")
    for c in cands:
        if (c / "model" / "renderer" / "msplat.py").is_file():
            return c
    return None


def examples_dir() -> Path | None:
    """Directory holding the reference's ``examples/supervise/renderer.py``
    (the normal-feature renderer), or None."""
    root = pointrix_dir()
    if root is None:
        return None
    for c in (root.parent / "examples" / "supervise", root.parent.parent / "examples" / "supervise"):
        if (c / "renderer.py").is_file():
            return c
    return None


# ------------------------------------------------------------------ stubs ---
def _stub_module(name: str, **attrs) -> types.ModuleType:
    """A module with a spec, so that ``importlib.util.find_spec`` (which torch
    calls on some module names) treats it like any loaded module."""
    m = types.ModuleType(name)
    m.__spec__ = importlib.machinery.ModuleSpec(name, None)
    m.__dict__.update(attrs)
    return m


class _AnyIndex:
    """``Float[Tensor, "N 3"]`` and the like: annotations only."""

    def __getitem__(self, item):
        return object


class _Registry:
    def __init__(self, name, modules=None):
        self._name = name
        self._obj_map = {}

    def register(self, obj=None):
        def deco(o):
            self._obj_map[o.__name__] = o
            return o
        return deco(obj) if obj is not None else deco

    def get(self, name):
        return self._obj_map[name]


class _BaseObject:
    class Config:
        pass

    def __init__(self, cfg=None, *args, **kwargs):
        conf = self.Config
        if cfg is None:
            self.cfg = conf()
        elif isinstance(cfg, dict) and is_dataclass(conf):
            self.cfg = conf(**cfg)
        else:
            self.cfg = cfg
        self.device = "cuda"
        self.setup(*args, **kwargs)

    def setup(self, *args, **kwargs):
        pass


def _schedule_c(value, epoch, global_step):
    if isinstance(value, (int, float)):
        return value
    raise TypeError("schedule lists are not needed by the statistics under test")


def _install_stubs(root: Path) -> None:
    if "pointrix" in sys.modules and getattr(sys.modules["pointrix"], "_pgb_ref_root", None) == str(root):
        return
    for mod in [k for k in sys.modules if k == "pointrix" or k.startswith("pointrix.")]:
        del sys.modules[mod]
    for name in ("jaxtyping", "lpips"):
        try:
            __import__(name)
        except Exception:
            sys.modules[name] = _stub_module(name, Float=_AnyIndex(), Int=_AnyIndex(),
                                             Bool=_AnyIndex())
    try:
        __import__("sklearn.neighbors")
    except Exception:
        sys.modules["sklearn"] = _stub_module("sklearn")
        sys.modules["sklearn.neighbors"] = _stub_module("sklearn.neighbors", NearestNeighbors=object)
    # synthetic packages whose __path__ is the reference's directories, so that
    # relative imports inside the reference files resolve to the real files
    for pkg in ("", ".model", ".model.renderer", ".model.renderer.utils", ".model.utils",
                ".utils", ".controller"):
        name = "pointrix" + pkg
        m = _stub_module(name)
        m.__path__ = [str(root / pkg[1:].replace(".", "/"))] if pkg else [str(root)]
        m.__spec__.submodule_search_locations = list(m.__path__)
        m.__package__ = name
        sys.modules[name] = m
    sys.modules["pointrix"]._pgb_ref_root = str(root)
    sys.modules["pointrix.utils.base"] = _stub_module("pointrix.utils.base", BaseObject=_BaseObject)
    sys.modules["pointrix.utils.registry"] = _stub_module("pointrix.utils.registry",
                                                          Registry=_Registry)
    sys.modules["pointrix.utils.config"] = _stub_module("pointrix.utils.config", C=_schedule_c)


def _load_file(name: str, path: Path, bind: dict | None = None) -> types.ModuleType:
    """Executes ``path`` as module ``name``; ``bind`` maps top-level module
    names to module objects that its ``import`` statements must resolve to
    while it loads (e.g. ``msplat``)."""
    spec = importlib.util.spec_from_file_location(name, str(path))
    mod = importlib.util.module_from_spec(spec)
    saved = {}
    for k, v in (bind or {}).items():
        saved[k] = sys.modules.get(k)
        sys.modules[k] = v
    try:
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    return mod


def _module(dotted: str) -> types.ModuleType | None:
    root = pointrix_dir()
    if root is None:
        return None
    _install_stubs(root)
    name = "pointrix." + dotted
    if name in sys.modules and getattr(sys.modules[name], "__file__", None):
        return sys.modules[name]
    return _load_file(name, root / (dotted.replace(".", "/") + ".py"))


def renderer_utils():
    """``pointrix/model/renderer/utils/renderer_utils.py`` (RenderFeatures)."""
    return _module("model.renderer.utils.renderer_utils")


def pose():
    """``pointrix/utils/pose.py`` (unitquat_to_rotmat, quat_to_rotmat)."""
    return _module("utils.pose")


def loss():
    """``pointrix/model/loss.py`` (ssim, l1_loss, l2_loss)."""
    return _module("model.loss")


def gs_controller():
    """``pointrix/controller/gs.py`` (DensificationController)."""
    _module("controller.base")
    return _module("controller.gs")


def msplat_renderer(msplat_module) -> types.ModuleType | None:
    """``pointrix/model/renderer/msplat.py`` executed with its ``import
    msplat`` bound to ``msplat_module`` (the GB300 shim, or the oracle's CPU
    operators).  A fresh module object per call."""
    root = pointrix_dir()
    if root is None:
        return None
    _install_stubs(root)
    renderer_utils()
    tag = getattr(msplat_module, "__name__", "msplat").replace(".", "_")
    return _load_file(f"pointrix.model.renderer.msplat_{tag}", root / "model/renderer/msplat.py",
                      bind={"msplat": msplat_module})


def normal_renderer(msplat_module) -> types.ModuleType | None:
    """``examples/supervise/renderer.py`` (MsplatNormalRender, rgb + normal
    features), subclassing the reference ``MsplatRender``, with ``msplat``
    bound as above; None when the example file is not installed."""
    ex = examples_dir()
    if ex is None:
        return None
    base = msplat_renderer(msplat_module)
    shim = _stub_module("pointrix.model.renderer.msplat", MsplatRender=base.MsplatRender,
                        RENDERER_REGISTRY=base.RENDERER_REGISTRY)
    tag = getattr(msplat_module, "__name__", "msplat").replace(".", "_")
    return _load_file(f"pgb_ref_examples_supervise_renderer_{tag}", ex / "renderer.py",
                      bind={"msplat": msplat_module, "pointrix.model.renderer.msplat": shim})


def make_render(module, render_depth=False, max_sh_degree=3, white_bg=False, cls="MsplatRender"):
    """An instance of the reference renderer class ``cls`` from ``module``,
    built as Pointrix builds it (``cfg`` dict, then ``setup(white_bg,
    device)``)."""
    klass = getattr(module, cls)
    return klass({"render_depth": render_depth, "max_sh_degree": max_sh_degree}, white_bg,
                 "cuda")


@contextlib.contextmanager
def cuda_calls_stay_on_cpu():
    """``render_iter`` moves ``position`` with ``.cuda()``
    (``pointrix/model/renderer/msplat.py:94-95``); on a host without a GPU the
    CPU fixtures are made with that call returning the tensor itself."""
    import torch

    orig = torch.Tensor.cuda
    torch.Tensor.cuda = lambda self, *a, **k: self
    try:
        yield
    finally:
        torch.Tensor.cuda = orig
