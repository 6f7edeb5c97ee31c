"""Helpers for the GPU tests: device buffers (torch) around the stage-level C ABI."""
import math

import numpy as np

from gs300 import records as R
from gs300 import scene as S


def frame_psnr(a, b):
    d = a[..., :3].astype(np.float64) - b[..., :3].astype(np.float64)
    mse = (d ** 2).mean()
    return math.inf if mse == 0 else 10.0 * math.log10(255.0 ** 2 / mse)


def within_one_fraction(a, b):
    d = np.abs(a.astype(np.int32) - b.astype(np.int32)).max(axis=-1)
    return float((d <= 1).mean())


def uniforms(gs, w, h, k=0, mode=R.DISPLAY_SPLAT, radius=8.0, mt=None, sh_deg=3, no_sh0=False, std=3.0, size=1.0, camera=None):
    cam = camera if camera is not None else S.orbit_camera(k, radius=radius)
    pod = gs.CameraPod.new(cam, (w, h))
    gt = gs.gaussian_transform_pod(size, mode, sh_deg, no_sh0, std)
    return gs.frame_uniforms(pod, mt if mt is not None else gs.model_transform_pod(), gt, (w, h))


class StagePipeline:
    """Preprocess -> sort -> rasterise through the stage entry points, on caller buffers."""

    def __init__(self, gs, torch, records, fmt, w, h, max_pairs=None):
        self.gs, self.torch = gs, torch
        self.n = len(records)
        self.fmt = fmt
        dev = "cuda"
        raw = np.frombuffer(records.tobytes(), np.uint8)
        self.records = torch.from_numpy(raw.copy()).to(dev) if raw.size else torch.zeros(16, dtype=torch.uint8, device=dev)
        n = max(self.n, 1)
        self.control = torch.zeros(8, dtype=torch.int32, device=dev)
        self.indices = torch.zeros(n, dtype=torch.int32, device=dev)
        self.depth_cap = gs.Preprocessor.depth_capacity(self.n)
        self.depths = torch.zeros(max(self.depth_cap, 1), dtype=torch.float32, device=dev)
        self.splats = torch.zeros(n * 12, dtype=torch.float32, device=dev)
        self.pre_bytes = gs.Preprocessor.scratch_bytes(self.n)
        self.pre_scratch = torch.zeros(self.pre_bytes, dtype=torch.uint8, device=dev)
        self.sort_bytes = gs.RadixSorter.scratch_bytes(self.n)
        self.sort_scratch = torch.zeros(self.sort_bytes, dtype=torch.uint8, device=dev)
        self.w, self.h = w, h
        self.max_pairs = max_pairs or (8 * self.n + 4096)
        self.r_bytes = gs.Renderer.scratch_bytes(self.n, w, h, self.max_pairs)
        self.r_scratch = torch.zeros(self.r_bytes, dtype=torch.uint8, device=dev)
        self.target = torch.zeros((h, w, 4), dtype=torch.uint8, device=dev)

    def preprocess(self, u, selection=None, invert=False):
        gs = self.gs
        sel = None if selection is None else self.torch.from_numpy(np.ascontiguousarray(selection, np.uint32).view(np.int32)).cuda()
        gs.Preprocessor.preprocess(u, self.records, self.fmt, self.n, self.control, self.control.data_ptr() + 16, self.indices,
                                   self.depths, self.depth_cap, self.splats, self.pre_scratch, self.pre_bytes, selection=sel,
                                   invert_selection=invert)

    def sort(self):
        self.gs.RadixSorter.sort(self.depths, self.indices, self.n, self.sort_scratch, self.sort_bytes,
                                 count=self.control.data_ptr() + 4)

    def rasterize(self, u):
        self.gs.Renderer.render(u, self.splats, self.indices, self.control.data_ptr() + 4, self.n, self.target, self.w, self.h,
                                self.w * 4, self.max_pairs, self.r_scratch, self.r_bytes)

    def render(self, u):
        self.preprocess(u)
        self.sort()
        self.rasterize(u)
        self.torch.cuda.synchronize()
        return self.frame()

    def count(self):
        return int(self.control[1].item())

    def frame(self):
        return self.target.cpu().numpy()

    def splat_records(self):
        return self.splats.cpu().numpy().view(R.SPLAT_DTYPE)[: self.n]
