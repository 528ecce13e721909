"""Camera (camera.rs:21-160): observer tetrad on the GPU, pixel ray states."""
import numpy as np

from . import _ffi
from ._util import check, dp, f64


class Camera:
    """Camera::new(observer, fov_y_deg, width, height). forward_sign=+1 is the
    reference camera (forward = -e1); -1 looks along +e1 (an extension)."""

    def __init__(self, observer, fov_y_deg, width, height, forward_sign=1):
        self.observer = f64(observer, (4,))
        self.fov_y_deg = float(fov_y_deg)
        self.fov_y_rad = self.fov_y_deg * (np.pi / 180.0)
        self.width = int(width)
        self.height = int(height)
        self.forward_sign = int(forward_sign)

    @classmethod
    def new(cls, observer, fov_y_deg, width, height):
        return cls(observer, fov_y_deg, width, height)

    def c_struct(self):
        c = _ffi.GeonCamera()
        for i in range(4):
            c.observer[i] = float(self.observer[i])
        c.fov_y_deg = self.fov_y_deg
        c.width = self.width
        c.height = self.height
        c.forward_sign = self.forward_sign
        return c

    def tetrad(self, metric):
        """Camera::tetrad (camera.rs:47-97): rows are e_(a)^mu."""
        out = np.empty(16)
        check(_ffi.load().geon_camera_tetrad(metric.handle, dp(self.observer), dp(out)))
        return out.reshape(4, 4)

    def ray_states(self, tetrad, du=0.5, dv=0.5):
        """Camera::ray_state_sub for every pixel: (height*width, 8), row-major."""
        c = self.c_struct()
        t = f64(tetrad, (16,))
        out = np.empty((self.width * self.height, 8))
        check(_ffi.load().geon_camera_ray_states(c, dp(t), float(du), float(dv), dp(out)))
        return out

    def ray_state_sub(self, tetrad, i, j, du, dv):
        return self.ray_states(tetrad, du, dv)[j * self.width + i]

    def ray_state(self, tetrad, i, j):
        return self.ray_state_sub(tetrad, i, j, 0.5, 0.5)
