"""sphere_stereo_gb300: GB300-native (sm_103a) sphere-sweeping stereo, a drop-in for the
per-frame path of KAIST-VCLAB/sphere-stereo (python/depth_estimation.py, python/isb_filter.py,
python/stitcher.py, python/utils.py).

The directory name is not a Python identifier; import it with
``importlib.import_module("sphere-stereo_gb300")`` (the repository root on ``sys.path``).
The public names mirror the reference's modules; the compute runs in libsphere_stereo_gb300.so
(C ABI: include/sphere_stereo_gb300.h), built by ``_build.build()``.
"""
from . import _native
from .depth_estimation import RGBD_Estimator, distance_candidates
from .differentiable import DifferentiableSweep
from .isb_filter import ISB_Filter
from .stitcher import Stitcher, vectorize_calibration
from .utils import Calibration, parse_json_calib, project, rgb2yCbCr, rgb_to_guide, unproject

__all__ = ["RGBD_Estimator", "ISB_Filter", "Stitcher", "Calibration", "parse_json_calib", "unproject", "project",
           "rgb2yCbCr", "rgb_to_guide", "vectorize_calibration", "distance_candidates", "DifferentiableSweep"]
