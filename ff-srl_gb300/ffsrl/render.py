"""WarpRaycastRendererDO: BVH ray-cast of every environment (reference
``FF_SRL/FF_SRL/render.py:826-1196``).

``renderNew(simBVH, simModel)`` returns the per-env images ``[N, R, R, 3]`` as a device
tensor (the reference's ``wp.to_torch(pixels).view(N, R, R, 3)``, ``render.py:1113``).
Each pixel averages 2x2 rays (``num_samples = 1`` -> rays of ``2R x 2R``).  One pass
writes the colour image in ``render_mode`` (``RenderMode``: grayscale, texture, normal
map, vertex colour or depth map) into ``pixels`` and depth ``t/50`` (one channel) into
``depth``.

Display back-ends of the reference (matplotlib, terminal, OpenGL window) are not
available; every ``mode`` renders headless and returns the tensor.

Cameras: the reference shares one camera (``camera.pos[0]``, ``render.py:309``);
``setCameras`` gives each environment its own pose.
"""

from __future__ import annotations

import contextlib
import ctypes as C
import math
import warnings

import numpy as np
import torch

from . import _lib
from ._lib import check, lib, ptr


def quat_rpy(roll: float, pitch: float, yaw: float) -> np.ndarray:
    """Quaternion (x, y, z, w) of rotations roll about x, pitch about y, yaw about z."""
    cy, sy = math.cos(yaw * 0.5), math.sin(yaw * 0.5)
    cr, sr = math.cos(roll * 0.5), math.sin(roll * 0.5)
    cp, sp = math.cos(pitch * 0.5), math.sin(pitch * 0.5)
    w = cy * cr * cp + sy * sr * sp
    x = cy * sr * cp - sy * cr * sp
    y = cy * cr * sp + sy * sr * cp
    z = sy * cr * cp - cy * sr * sp
    return np.array([x, y, z, w], dtype=np.float32)


def look_at_rotation(pos, at) -> np.ndarray:
    """lookAt (render.py:1186-1196): pitch = asin(dir.y), yaw = atan2(dir.x, dir.z) - pi,
    rotation quat_rpy(pitch, yaw, 0)."""
    d = np.asarray(at, dtype=np.float64) - np.asarray(pos, dtype=np.float64)
    d = d / np.linalg.norm(d)
    pitch = math.asin(d[1])
    yaw = math.atan2(d[0], d[2]) - math.pi
    return quat_rpy(pitch, yaw, 0.0)


class RenderMode:
    """Shading of the colour image (render.py:17-25, drawSimBVHKernelManyEnvs render.py:350-409).

    grayscale, texture and vertex_color are Lambert-lit; texture falls back to the vertex
    colour for an env whose mesh has no texture; depth_map writes t/50 to all channels."""
    grayscale = 0
    texture = 1
    normal_map = 2
    vertex_color = 3
    depth_map = 4


class WarpRaycastRendererDO:
    def __init__(self, device, simModel, cameraPos=(3.0, 3.0, 3.0), cameraRot=(0.0, 0.0, 0.0),
                 lightPos=(3.0, 0.0, 0.0), lightIntensity=0.3, resolution: int = 512, mode: str = "human",
                 horizontalAperture: float = 19.2, verticalAperture: float = 19.2, fused: bool = True,
                 render_mode: int = RenderMode.texture):
        if mode not in ("headless", "gpuless"):
            warnings.warn(f"render mode {mode!r}: no display back-end here, rendering headless")
        self.device = torch.device(device)
        self.mode = mode
        self.simModel = simModel
        self.numEnvs = simModel.numEnvs
        self.fused = bool(fused)
        if int(render_mode) not in range(5):
            raise ValueError(f"render_mode {render_mode!r}: expected a RenderMode value 0..4")
        self.render_mode = int(render_mode)  # the reference's default is RenderMode.texture (render.py:852)
        self.height = self.width = int(resolution)
        self.num_pixels = self.width * self.height
        self.num_samples = 1
        self.rays_width = self.width * 2 ** self.num_samples
        self.rays_height = self.height * 2 ** self.num_samples
        self.num_rays = self.rays_width * self.rays_height
        self.cameraPos = np.asarray(cameraPos, dtype=np.float32)
        self.cameraRot = np.asarray(cameraRot, dtype=np.float32)
        focal = 50.0
        self.camera_tan = verticalAperture / (2.0 * focal)
        self.camera_aspect = horizontalAperture / verticalAperture
        f32 = dict(dtype=torch.float32, device=self.device)
        self.cameraPosT = torch.as_tensor(self.cameraPos.reshape(1, 3), **f32).clone()
        self.cameraRotT = torch.as_tensor(quat_rpy(self.cameraRot[2], self.cameraRot[0], self.cameraRot[1]).reshape(1, 4),
                                          **f32).clone()
        self.lightDir = torch.as_tensor(np.asarray([lightPos], dtype=np.float32), **f32)
        self.lightIntensity = torch.as_tensor(np.asarray([lightIntensity], dtype=np.float32), **f32)
        N, R = self.numEnvs, self.width
        self.pixels = torch.zeros((N * R * R, 3), **f32)
        self.depth = torch.zeros(N * R * R, **f32)
        self.meshNormalSums = torch.zeros((simModel.numAllVisPoints, 3), **f32)
        self.vertexNormals = torch.zeros((simModel.numAllVisPoints, 3), **f32)
        self.errorFlag = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.rays = None
        self.rayDepth = None
        # point -> incident faces (ascending face id) for the deterministic normal gather
        faces = simModel.host["allVisFace"].reshape(-1, 3).astype(np.int64)
        P = simModel.numAllVisPoints
        pts = faces.reshape(-1)
        fid = np.repeat(np.arange(len(faces)), 3)
        order = np.lexsort((fid, pts))
        counts = np.bincount(pts, minlength=P)
        self.pointFaceStart = torch.as_tensor(np.concatenate([[0], np.cumsum(counts)]).astype(np.int32),
                                              dtype=torch.int32, device=self.device)
        self.pointFace = torch.as_tensor(fid[order].astype(np.int32), dtype=torch.int32, device=self.device)
        self.renderGraph = None

    def setCameras(self, pos, rot) -> None:
        """Per-env cameras: pos [N, 3], rot [N, 4] quaternions (x, y, z, w)."""
        f32 = dict(dtype=torch.float32, device=self.device)
        self.cameraPosT = torch.as_tensor(np.asarray(pos, dtype=np.float32).reshape(-1, 3), **f32).clone()
        self.cameraRotT = torch.as_tensor(np.asarray(rot, dtype=np.float32).reshape(-1, 4), **f32).clone()

    def lookAt(self, at) -> None:
        """Point the shared camera at ``at`` (render.py:1186-1196)."""
        q = look_at_rotation(self.cameraPos, at)
        self.cameraRotT = torch.as_tensor(q.reshape(1, 4), dtype=torch.float32, device=self.device).clone()

    def _desc(self, simModel) -> _lib.Render:
        r = _lib.Render()
        r.num_envs, r.resolution = self.numEnvs, self.width
        r.num_vis_points, r.num_vis_faces = simModel.numAllVisPoints, simModel.numAllVisFaces
        r.vis_point, r.vis_face = ptr(simModel.allVisPoint), ptr(simModel.allVisFace)
        r.vis_point_color = ptr(simModel.allVisPointColor)
        r.normal_sum, r.vertex_normal = ptr(self.meshNormalSums), ptr(self.vertexNormals)
        r.point_face_start, r.point_face = ptr(self.pointFaceStart), ptr(self.pointFace)
        r.num_cameras = int(self.cameraPosT.shape[0])
        r.camera_pos, r.camera_rot = ptr(self.cameraPosT), ptr(self.cameraRotT)
        r.camera_tan, r.camera_aspect = self.camera_tan, self.camera_aspect
        r.num_lights = int(self.lightDir.shape[0])
        r.light_dir, r.light_intensity = ptr(self.lightDir), ptr(self.lightIntensity)
        r.color, r.depth = ptr(self.pixels), ptr(self.depth)
        if not self.fused:
            if self.rays is None:
                self.rays = torch.zeros((self.numEnvs * self.num_rays, 3), dtype=torch.float32, device=self.device)
                self.rayDepth = torch.zeros(self.numEnvs * self.num_rays, dtype=torch.float32, device=self.device)
            r.rays, r.ray_depth = ptr(self.rays), ptr(self.rayDepth)
        r.error_flag = ptr(self.errorFlag)
        r.env_point_start = ptr(simModel.envVisPointStartT)
        r.render_mode = int(self.render_mode)
        if simModel.hasTextures:
            r.texture, r.tex_coords, r.tex_indices = ptr(simModel.textureT), ptr(simModel.texCoordsT), \
                ptr(simModel.texIndicesT)
            r.env_objects, r.object_texture = ptr(simModel.envObjectsT), ptr(simModel.objectTextureT)
        return r

    def renderFunctionNew(self, simBVH, stream=None) -> None:
        self.simModel.require_cuda()
        r = self._desc(self.simModel)
        fn = lib().ffsrl_render_fused if self.fused else lib().ffsrl_render_reference
        check(fn(C.byref(r), C.byref(simBVH.desc), _lib.stream_handle(stream)))

    def renderNew(self, simBVH, simModel, stream=None, useGraph: bool = False) -> torch.Tensor:
        """Images [N, R, R, 3] (render.py:1099-1113).  ``useGraph`` captures the render
        into a CUDA graph on the first call and replays it afterwards, as the reference's
        ``renderGraph``; a new graph is captured when the BVH, shading mode, path or camera
        tensors change."""
        if useGraph:
            from .graphs import Graph
            key = (id(simBVH), self.render_mode, self.fused, self.cameraPosT.data_ptr(), self.cameraRotT.data_ptr(),
                   self.lightDir.data_ptr())
            if self.renderGraph is None or self.renderGraph[0] != key:
                self.renderGraph = (key, Graph(lambda: self.renderFunctionNew(simBVH),
                                               prepare=lambda: self._desc(self.simModel)))
            with torch.cuda.stream(stream) if stream is not None else contextlib.nullcontext():
                self.renderGraph[1]()
        else:
            self.renderFunctionNew(simBVH, stream)
        return self.pixels.view(self.numEnvs, self.height, self.width, 3)

    def depthImages(self) -> torch.Tensor:
        return self.depth.view(self.numEnvs, self.height, self.width)

    def checkErrors(self) -> None:
        """Raises if a ray exhausted its traversal stack since the last check."""
        if int(self.errorFlag.item()) != 0:
            self.errorFlag.zero_()
            raise _lib.FFSRLError(_lib.ERR_STACK_OVERFLOW, "BVH traversal stack overflow")
