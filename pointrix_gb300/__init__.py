"""GB300-native (sm_103a) implementation of the msplat operators behind
Pointrix's ``MsplatRender``: projection, 3D covariance, EWA conic, SH colour,
tile binning/sort and alpha blending, each with its backward."""
from .ops import (  # noqa: F401
    EXTENT_DEFAULT,
    NEAREST_DEFAULT,
    alpha_blending,
    alpha_blending_with_state,
    check_device_status,
    compute_cov3d,
    compute_sh,
    ewa_project,
    project_point,
    sort_gaussian,
)
from ._lib import PgbError  # noqa: F401

__version__ = "0.1.0"
