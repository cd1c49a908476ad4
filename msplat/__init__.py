"""Drop-in ``msplat`` module: Pointrix's ``import msplat``
(``pointrix/model/renderer/msplat.py:2``) resolves to the GB300 operators."""
from pointrix_gb300.ops import (  # noqa: F401
    alpha_blending,
    compute_cov3d,
    compute_sh,
    ewa_project,
    project_point,
    sort_gaussian,
)
