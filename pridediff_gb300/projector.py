"""Projector modules: drop-in for deeprecon.torch.projector.

``projector2d``, ``projector3d`` and ``projectorsp`` keep deeprecon's
constructor signatures, defaults, options packing, arc conversion, shape
assertions and method names (deeprecon/deeprecon/torch/projector/
projector.py:55-563); the operators dispatch to the autograd pairs in
``function.py`` and from there to ``libpridediff_dd.so``.

Options packing (the order every kernel reads):
  2-D  [W, H, D, sx, sy, det_size, iso_source, source_detector, px, py, bin]
  3-D  [W, H, Dep, C, R, sx, sy, sz, dc, dr, iso_source, source_detector,
        px, py, pz, bin_c, bin_r]
  sp   the 3-D list without pz (16 entries)
For arc detectors the column pitch and shift are divided by the
source-detector distance (angles), as the reference does.
"""
from __future__ import annotations

from typing import List, Tuple, Union

import torch
import torch.nn as nn
from torch import Tensor

from . import fbp
from . import function as F
from .filter import filter_generate

__functions__ = {
    "dis": {
        "flat": {
            "projection": F.ProjFanFlatDis2d, "projection_t": F.ProjTransFanFlatDis2d,
            "bprojection": F.BackProjFanFlatDis2d, "bprojection_t": F.BackProjTransFanFlatDis2d,
            "bprojection_w": F.BackProjWeightedFanFlatDis2d, "get_sys_matrix": F.GetSysMatrixFanFlat2d,
            "projection3d": F.ProjConeFlatDis3d, "projection3d_t": F.ProjTransConeFlatDis3d,
            "bprojection3d": F.BackProjConeFlatDis3d, "bprojection3d_t": F.BackProjTransConeFlatDis3d,
            "bprojection3d_w": F.BackProjWeightedConeFlatDis3d,
        },
        "arc": {
            "projection": F.ProjFanArcDis2d, "projection_t": F.ProjTransFanArcDis2d,
            "bprojection": F.BackProjFanArcDis2d, "bprojection_t": F.BackProjTransFanArcDis2d,
            "bprojection_w": F.BackProjWeightedFanArcDis2d, "get_sys_matrix": F.GetSysMatrixFanArc2d,
            "projection3d": F.ProjConeArcDis3d, "projection3d_t": F.ProjTransConeArcDis3d,
            "bprojection3d": F.BackProjConeArcDis3d, "bprojection3d_t": F.BackProjTransConeArcDis3d,
            "bprojection3d_w": F.BackProjWeightedConeArcDis3d,
            "projectionsp": F.ProjSpiralDis3d, "projectionsp_t": F.ProjTransSpiralDis3d,
            "bprojectionsp": F.BackProjSpiralDis3d, "bprojectionsp_t": F.BackProjTransSpiralDis3d,
            "bprojectionsp_w": F.BackProjWeightedSpiralDis3d,
        },
        "para": {
            "projection": F.ProjParaDis2d, "projection_t": F.ProjTransParaDis2d,
            "bprojection": F.BackProjParaDis2d, "bprojection_t": F.BackProjTransParaDis2d,
            # the parallel beam has no weighted variant (projector.py:49)
            "bprojection_w": F.BackProjParaDis2d, "get_sys_matrix": F.GetSysMatrixPara2d,
        },
    }
}


def _tuple(x, n, what):
    if not isinstance(x, (tuple, list)):
        x = (x,) * n
    assert len(x) == n, what
    return tuple(x)


class projector2d(nn.Module):
    r"""2-D distance-driven projector (parallel, fan-flat, fan-arc).

    Args as deeprecon's projector2d: image_size (int or (width, height)),
    num_det, pix_size (float or (sx, sy)), det_size, iso_source,
    source_detector, pixshift=0., binshift=0., scan_type='flat'
    ('flat'|'arc'|'para'), method='dis', filter_type='ramp'
    ('ramp'|'sheeplogan'), trainable=False, dtype=None.
    """

    def __init__(self, image_size: Union[int, Tuple[int], List[int]], num_det: int,
                 pix_size: Union[float, Tuple[float], List[float]], det_size: float,
                 iso_source: float, source_detector: float,
                 pixshift: Union[float, Tuple[float], List[float]] = 0., binshift: float = 0.,
                 scan_type: str = "flat", method: str = "dis", filter_type: str = "ramp",
                 trainable: bool = False, dtype=None) -> None:
        super().__init__()
        image_size = _tuple(image_size, 2, "Image resolution should be a int or two-tuple int")
        pix_size = _tuple(pix_size, 2, "Pixle size should be a float or two-tuple float")
        pixshift = _tuple(pixshift, 2, "Scanned object shift should be a float or two-tuple float")
        scan_type, method, filter_type = scan_type.lower(), method.lower(), filter_type.lower()
        assert scan_type in {"flat", "arc", "para"}, f"Scanning mode {scan_type} not supported"
        assert method in {"dis"}, f"Radon transform method {method} not supported"
        if scan_type == "arc":
            det_size = det_size / source_detector
            binshift = binshift / source_detector
        options = torch.tensor([*image_size, num_det, *pix_size, det_size, iso_source,
                                source_detector, *pixshift, binshift], dtype=dtype)
        self.image_size = tuple(image_size)
        self.num_det = num_det
        self.det_size = det_size
        self.binshift = binshift
        self.iso_source = iso_source
        self.source_detector = source_detector
        self.scan_type = scan_type
        self.method = method
        self.filter_type = filter_type
        self.options = nn.parameter.Parameter(options, requires_grad=False)
        self.filter = nn.parameter.Parameter(self.filter_generate(self.filter_type, dtype=dtype),
                                             requires_grad=trainable)
        self.weight = nn.parameter.Parameter(self.weight_generate(dtype=dtype), requires_grad=trainable)

    def _fn(self, key):
        return __functions__[self.method][self.scan_type][key]

    def _check_image(self, image):
        b, c, h, w = image.shape
        assert (w, h) == self.image_size, "The size of input image is inconsistent with geometry"

    def _check_sino(self, sino, angles):
        b, c, h, w = sino.shape
        v, = angles.shape
        assert (h, w) == (v, self.num_det), "The size of input sinogram is inconsistent with geometry"

    def projection(self, image: Tensor, angles: Tensor) -> Tensor:
        self._check_image(image)
        return self._fn("projection").apply(image, self.options, angles)

    def backprojection(self, sino: Tensor, angles: Tensor) -> Tensor:
        self._check_sino(sino, angles)
        return self._fn("bprojection").apply(sino, self.options, angles)

    def backprojection_w(self, sino: Tensor, angles: Tensor) -> Tensor:
        self._check_sino(sino, angles)
        return self._fn("bprojection_w").apply(sino, self.options, angles)

    def projection_t(self, sino: Tensor, angles: Tensor) -> Tensor:
        self._check_sino(sino, angles)
        return self._fn("projection_t").apply(sino, self.options, angles)

    def backprojection_t(self, image: Tensor, angles: Tensor) -> Tensor:
        self._check_image(image)
        return self._fn("bprojection_t").apply(image, self.options, angles)

    def forward(self, image: Tensor, angles: Tensor) -> Tensor:
        return self.projection(image, angles)

    def filter_generate(self, filter_type, dtype=None):
        det = self.det_size * self.iso_source / self.source_detector if self.scan_type == "flat" else self.det_size
        return filter_generate(self.num_det, det, filter_type, dtype)[None, None, None, :]

    def weight_generate(self, dtype=None):
        u = torch.arange((-self.num_det / 2 + 0.5), self.num_det / 2, 1, dtype=dtype)
        u = u * self.det_size + self.binshift
        if self.scan_type == "flat":
            u = u * self.iso_source / self.source_detector
            return self.iso_source / torch.sqrt(u ** 2 + self.iso_source ** 2)
        if self.scan_type == "arc":
            return torch.cos(u)
        return torch.ones_like(u)

    def filtered_backprojection(self, sino: Tensor, angles: Tensor, filter: Union[Tensor, None] = None,
                                filter_type: Union[str, None] = None, redundant: bool = True) -> Tensor:
        if filter is not None:
            taps = filter
        elif filter_type is None or filter_type.lower() == self.filter_type:
            taps = self.filter
        else:
            taps = self.filter_generate(filter_type.lower(), dtype=sino.dtype).to(sino.device)
        if fbp.fused_ok(sino, self.weight, taps):
            filtered = fbp.weighted_filter(sino, self.weight, taps)
        else:   # a trainable weight or filter: autograd through the torch convolution
            filtered = nn.functional.conv2d(sino * self.weight, taps, padding=(0, self.num_det - 1))
        recon = self.backprojection_w(filtered, angles)
        recon = recon * (angles[-1] - angles[0]).abs() / (angles.size(0) - 1)
        if redundant:
            recon = recon / 2
        return recon

    def get_sys_matrix(self, angles: Tensor) -> Tensor:
        return self._fn("get_sys_matrix")(self.options, angles)


class projector3d(nn.Module):
    r"""3-D cone-beam distance-driven projector ('flat' or 'arc' detector).

    Args as deeprecon's projector3d: image_size (int or (W, H, Dep)),
    num_det (int or (col, row)), pix_size, det_size ((col, row)), iso_source,
    source_detector, pixshift (3), binshift (2), scan_type='flat',
    method='dis', filter_type='ramp', trainable=False, dtype=None.
    """

    def __init__(self, image_size, num_det, pix_size, det_size, iso_source: float,
                 source_detector: float, pixshift=0., binshift=0., scan_type: str = "flat",
                 method: str = "dis", filter_type: str = "ramp", trainable: bool = False,
                 dtype=None) -> None:
        super().__init__()
        image_size = _tuple(image_size, 3, "Image resolution should be a int or three-tuple int")
        num_det = _tuple(num_det, 2, "Number of detector elements should be a int or two-tuple int")
        pix_size = _tuple(pix_size, 3, "Pixle size should be a float or three-tuple float")
        det_size = _tuple(det_size, 2, "The size of detector element should be a float or two-tuple float")
        pixshift = _tuple(pixshift, 3, "Scanned object shift should be a float or three-tuple float")
        binshift = _tuple(binshift, 2, "Detector shift should be a float or two-tuple float")
        scan_type, method, filter_type = scan_type.lower(), method.lower(), filter_type.lower()
        assert scan_type in {"flat", "arc"}, f"Scanning mode {scan_type} not supported"
        assert method in {"dis"}, f"Radon transform method {method} not supported"
        if scan_type == "arc":
            det_size = (det_size[0] / source_detector, det_size[1])
            binshift = (binshift[0] / source_detector, binshift[1])
        options = torch.tensor([*image_size, *num_det, *pix_size, *det_size, iso_source,
                                source_detector, *pixshift, *binshift], dtype=dtype)
        self.image_size = tuple(image_size)
        self.num_det = tuple(num_det)
        self.det_size = det_size
        self.binshift = binshift
        self.iso_source = iso_source
        self.source_detector = source_detector
        self.scan_type = scan_type
        self.method = method
        self.filter_type = filter_type
        self.options = nn.parameter.Parameter(options, requires_grad=False)
        self.filter = nn.parameter.Parameter(self.filter_generate(self.filter_type, dtype=dtype),
                                             requires_grad=trainable)
        self.weight = nn.parameter.Parameter(self.weight_generate(dtype=dtype), requires_grad=trainable)

    _suffix = "3d"

    def _fn(self, key):
        return __functions__[self.method][self.scan_type][key]

    def _check_image(self, image):
        b, c, d, h, w = image.shape
        assert (w, h, d) == self.image_size, "The size of input image is inconsistent with geometry"

    def _check_sino(self, sino, angles):
        b, c, d, h, w = sino.shape
        v, = angles.shape
        assert (d, w, h) == (v, *self.num_det), "The size of input sinogram is inconsistent with geometry"

    def projection(self, image: Tensor, angles: Tensor) -> Tensor:
        self._check_image(image)
        return self._fn("projection3d").apply(image, self.options, angles)

    def backprojection(self, sino: Tensor, angles: Tensor) -> Tensor:
        self._check_sino(sino, angles)
        return self._fn("bprojection3d").apply(sino, self.options, angles)

    def backprojection_w(self, sino: Tensor, angles: Tensor) -> Tensor:
        self._check_sino(sino, angles)
        return self._fn("bprojection3d_w").apply(sino, self.options, angles)

    def projection_t(self, sino: Tensor, angles: Tensor) -> Tensor:
        self._check_sino(sino, angles)
        return self._fn("projection3d_t").apply(sino, self.options, angles)

    def backprojection_t(self, image: Tensor, angles: Tensor) -> Tensor:
        self._check_image(image)
        return self._fn("bprojection3d_t").apply(image, self.options, angles)

    def forward(self, image: Tensor, angles: Tensor) -> Tensor:
        return self.projection(image, angles)

    def filter_generate(self, filter_type, dtype=None):
        det = self.det_size[0] * self.iso_source / self.source_detector if self.scan_type == "flat" \
            else self.det_size[0]
        return filter_generate(self.num_det[0], det, filter_type, dtype)[None, None, None, None, :]

    def weight_generate(self, dtype=None):
        col_size, row_size = self.det_size
        col_n, row_n = self.num_det
        col_s, row_s = self.binshift
        wr = torch.arange((-row_n / 2 + 0.5), row_n / 2, 1, dtype=dtype)
        wr = (wr * row_size + row_s) * self.iso_source / self.source_detector
        wc = torch.arange((-col_n / 2 + 0.5), col_n / 2, 1, dtype=dtype)
        wc = wc * col_size + col_s
        if self.scan_type == "flat":
            wc = wc * self.iso_source / self.source_detector
        elif self.scan_type == "arc":
            wc = torch.tan(wc) * self.iso_source
        wr = wr[:, None].repeat(1, col_n)
        wc = wc[None, :].repeat(row_n, 1)
        return self.iso_source / torch.sqrt(wr ** 2 + wc ** 2 + self.iso_source ** 2)

    def filtered_backprojection(self, sino: Tensor, angles: Tensor, filter: Union[Tensor, None] = None,
                                filter_type: Union[str, None] = None, redundant: bool = True) -> Tensor:
        if filter is not None:
            taps = filter
        elif filter_type is None or filter_type.lower() == self.filter_type:
            taps = self.filter
        else:
            taps = self.filter_generate(filter_type.lower(), dtype=sino.dtype).to(sino.device)
        if fbp.fused_ok(sino, self.weight, taps):
            filtered = fbp.weighted_filter(sino, self.weight, taps)
        else:   # a trainable weight or filter: autograd through the torch convolution
            filtered = nn.functional.conv3d(sino * self.weight, taps, padding=(0, 0, self.num_det[0] - 1))
        recon = self.backprojection_w(filtered, angles)
        recon = recon * (angles[-1] - angles[0]).abs() / (angles.size(0) - 1)
        if redundant:
            recon = recon / 2
        return recon


class projectorsp(nn.Module):
    r"""Spiral (helical) distance-driven projector, arc detector.

    Args as deeprecon's projectorsp; every method also takes ``source_pos``,
    a (4, V) table [axial position, radius shift, angle shift, axial shift].
    """

    def __init__(self, image_size, num_det, pix_size, det_size, iso_source: float,
                 source_detector: float, pixshift=0., binshift=0., scan_type: str = "arc",
                 method: str = "dis", filter_type: str = "ramp", trainable: bool = False,
                 dtype=None) -> None:
        super().__init__()
        image_size = _tuple(image_size, 3, "Image resolution should be a int or three-tuple int")
        num_det = _tuple(num_det, 2, "Number of detector elements should be a int or two-tuple int")
        pix_size = _tuple(pix_size, 3, "Pixle size should be a float or three-tuple float")
        det_size = _tuple(det_size, 2, "The size of detector element should be a float or two-tuple float")
        pixshift = _tuple(pixshift, 2, "Scanned object shift should be a float or three-tuple float")
        binshift = _tuple(binshift, 2, "Detector shift should be a float or two-tuple float")
        scan_type, method, filter_type = scan_type.lower(), method.lower(), filter_type.lower()
        assert scan_type in {"arc"}, f"Scanning mode {scan_type} not supported"
        assert method in {"dis"}, f"Radon transform method {method} not supported"
        det_size = (det_size[0] / source_detector, det_size[1])
        binshift = (binshift[0] / source_detector, binshift[1])
        options = torch.tensor([*image_size, *num_det, *pix_size, *det_size, iso_source,
                                source_detector, *pixshift, *binshift], dtype=dtype)
        self.image_size = tuple(image_size)
        self.num_det = tuple(num_det)
        self.det_size = det_size
        self.binshift = binshift
        self.iso_source = iso_source
        self.source_detector = source_detector
        self.scan_type = scan_type
        self.method = method
        self.filter_type = filter_type
        self.options = nn.parameter.Parameter(options, requires_grad=False)
        self.filter = nn.parameter.Parameter(self.filter_generate(self.filter_type, dtype=dtype),
                                             requires_grad=trainable)
        self.weight = nn.parameter.Parameter(projector3d.weight_generate(self, dtype=dtype),
                                             requires_grad=trainable)

    def _fn(self, key):
        return __functions__[self.method][self.scan_type][key]

    def _check(self, x, angles, source_pos, image: bool):
        b, c, d, h, w = x.shape
        v, = angles.shape
        m, n = source_pos.shape
        if image:
            assert (w, h, d) == self.image_size, "The size of input image is inconsistent with geometry"
        else:
            assert (d, w, h) == (v, *self.num_det), "The size of input sinogram is inconsistent with geometry"
        assert (m, n) == (4, v), "The size of angles and source position is not consistent"

    def projection(self, image: Tensor, angles: Tensor, source_pos: Tensor) -> Tensor:
        self._check(image, angles, source_pos, True)
        return self._fn("projectionsp").apply(image, self.options, angles, source_pos)

    def backprojection(self, sino: Tensor, angles: Tensor, source_pos: Tensor) -> Tensor:
        self._check(sino, angles, source_pos, False)
        return self._fn("bprojectionsp").apply(sino, self.options, angles, source_pos)

    def backprojection_w(self, sino: Tensor, angles: Tensor, source_pos: Tensor) -> Tensor:
        self._check(sino, angles, source_pos, False)
        return self._fn("bprojectionsp_w").apply(sino, self.options, angles, source_pos)

    def projection_t(self, sino: Tensor, angles: Tensor, source_pos: Tensor) -> Tensor:
        self._check(sino, angles, source_pos, False)
        return self._fn("projectionsp_t").apply(sino, self.options, angles, source_pos)

    def backprojection_t(self, image: Tensor, angles: Tensor, source_pos: Tensor) -> Tensor:
        self._check(image, angles, source_pos, True)
        return self._fn("bprojectionsp_t").apply(image, self.options, angles, source_pos)

    def forward(self, image: Tensor, angles: Tensor, source_pos: Tensor) -> Tensor:
        return self.projection(image, angles, source_pos)

    def filter_generate(self, filter_type, dtype=None):
        return filter_generate(self.num_det[0], self.det_size[0], filter_type, dtype)[None, None, None, None, :]

    def weight_generate(self, dtype=None):
        return projector3d.weight_generate(self, dtype)

    def filtered_backprojection(self, sino: Tensor, angles: Tensor, source_pos: Tensor,
                                filter_type: Union[str, None] = None) -> Tensor:
        if filter_type is None or filter_type.lower() == self.filter_type:
            taps = self.filter
        else:
            taps = self.filter_generate(filter_type.lower(), dtype=sino.dtype).to(sino.device)
        if fbp.fused_ok(sino, self.weight, taps):
            filtered = fbp.weighted_filter(sino, self.weight, taps)
        else:   # a trainable weight or filter: autograd through the torch convolution
            filtered = nn.functional.conv3d(sino * self.weight, taps, padding=(0, 0, self.num_det[0] - 1))
        recon = self.backprojection_w(filtered, angles, source_pos)
        return recon * abs(angles[1] - angles[0]) / 2
