"""Processor-shaped host interface mirroring Voreen's CPURaycaster /
SingleVolumeRaycaster surface over the C ABI.

Port names, property names, defaults and error behaviour follow the
reference so tests read like its processor code:
  ports       volumehandle.volumehandle, image.entrypoints, image.exitpoints,
              image.output                       (volumeraycaster.cpp:44-47)
  properties  samplingRate (2.0, 0.01..20), isoValue (0.5), compositing
              (dvr/mip/iso/mop/mida/fhp/fhn), gammaValue (MIDA, 0, -1..1),
              shading (none/phong), gradient (central-differences),
              classification (transfer-function / pre-integrated-cpu /
              pre-integrated-approximation; pre-integrated-gpu falls back to
              pre-integrated-cpu with an error, cpuraycaster.cpp:123-129),
              preIntegrationTableSize (deriveFromBitDepth = 0 / 256 / 512 /
              1024, cpuraycaster.cpp:51-74), interactionCoarseness (3,
              1..8) and interactionQuality (1.0, 0.01..1)
              (volumeraycaster.cpp:65-66),
              transferFunction (keys + domain + gamma + thresholds),
              lightPosition, lightAmbient, lightDiffuse, lightSpecular,
              materialShininess, applyLightAttenuation, lightAttenuation,
              camera                              (volumeraycaster.cpp:42-157,
                                                   volumerenderer.cpp:41-53)
  process()   fits the TF width to the volume's bit depth and, on first use,
              its domain to the volume's real-world min/max
              (transfuncpropertybase.cpp:134-174,
              transfunc1dkeysproperty.cpp:94-140), uploads the volume when the
              inport changes, renders into image.output. On a failure it logs
              an error and returns without output, as CPURaycaster::process does
              (cpuraycaster.cpp:125-146); `lastError` keeps the message.
              Pre-integration tables are cached per (step, size, mode), one
              at a time, like PreIntegrationTableMap's default size 1
              (preintegrationtablemap.cpp:59-95).
              process(interacting=True) renders as SingleVolumeRaycaster does
              in interaction mode (singlevolumeraycaster.cpp:253-256): at
              output size / interactionCoarseness (integer division) with the
              sampling rate times interactionQuality
              (VolumeRaycaster::getSamplingStepSize, volumeraycaster.cpp:312-322),
              then rescaled bilinearly to the output size
              (rescaleRendering, volumeraycaster.cpp:348-375). The coarse
              frame's rays go through the coarse pixel centres (analytic
              entry/exit at the coarse size).
  bricks      Volumes larger than device memory, with the streaming controls
              of Voreen's octree raycaster (SingleOctreeRaycasterCL,
              modules/opencl/processors/singleoctreeraycastercl.cpp:294-305):
              brickPoolPlacement ("device" / "host": the bricked volume in
              pinned host memory), brickBufferSizeMB (device brick cache;
              0 = as much as free device memory allows, the reference's 512 MB
              default is too small for a GB300), brickUploadBudgetMB (32, bricks
              gathered per frame), useLevelOfDetail (a half-resolution level
              stands in for bricks not in the cache) and useIterativeRefinement
              (true): after a frame that read bricks without a slot the
              processor sets `invalidated`, as the reference invalidates
              itself until no more bricks are uploaded
              (singleoctreeraycastercl.cpp:780-838, 880-894).
"""
from __future__ import annotations

import logging
from dataclasses import dataclass, field

import numpy as np

from . import (CLASSIFY_PREINTEGRATED, CLASSIFY_TF, DVR, EE_ANALYTIC, EE_BUFFERS, FHN, FHP, ISO, MIDA, MIP, MOP,
               OUT_RGBA32F, PLACE_DEVICE, PLACE_HOST, SHADE_NONE, SHADE_PHONG, Context, PreIntegrationTable,
               TransferFunction, Volume, VrcError,
               default_params, image_rescale, make_camera, render, sampling_step)

log = logging.getLogger("voreen.CudaRaycaster")

COMPOSITING = {"dvr": DVR, "mip": MIP, "iso": ISO, "mop": MOP, "mida": MIDA, "fhp": FHP, "fhn": FHN}
CLASSIFICATION = ("transfer-function", "pre-integrated-gpu", "pre-integrated-cpu", "pre-integrated-approximation")
PREINT_TABLE_SIZES = (0, 256, 512, 1024)
SHADING = {"none": SHADE_NONE, "phong": SHADE_PHONG}
PLACEMENT = {"device": PLACE_DEVICE, "host": PLACE_HOST}


@dataclass
class VolumeData:
    """What a VolumePort carries: voxels (Z, Y, X) plus the metadata the
    march uses (spacing, offset, real-world mapping)."""
    voxels: np.ndarray
    spacing: tuple = (1.0, 1.0, 1.0)
    offset: tuple = (0.0, 0.0, 0.0)
    rwm: tuple = (1.0, 0.0)


class Port:
    def __init__(self, name: str):
        self.name = name
        self.data = None

    def setData(self, d):
        self.data = d

    def getData(self):
        return self.data

    def hasData(self) -> bool:
        return self.data is not None

    def isConnected(self) -> bool:
        return self.data is not None


@dataclass
class TransFunc1DKeys:
    keys: list = field(default_factory=lambda: [(0.0, (0, 0, 0, 0)), (1.0, (255, 255, 255, 255))])
    domain: tuple = (0.0, 1.0)
    gamma: float = 1.0
    threshold: tuple = (0.0, 1.0)
    width: int = 256
    domain_fitted: bool = False


class CudaRaycaster:
    className = "CudaRaycaster"
    category = "Raycasting"

    def __init__(self, device: int = 0):
        self.volumeInport = Port("volumehandle.volumehandle")
        self.entryPort = Port("image.entrypoints")
        self.exitPort = Port("image.exitpoints")
        self.outport = Port("image.output")
        self.samplingRate = 2.0
        self.isoValue = 0.5
        self.compositing = "dvr"
        self.shading = "none"
        self.gradient = "central-differences"
        self.classification = "transfer-function"
        self.preIntegrationTableSize = 0
        self.gammaValue = 0.0
        self.interactionCoarseness = 3
        self.interactionQuality = 1.0
        # proxy geometry of the analytic entry/exit (OptimizedProxyGeometry
        # "enableClipping" / "clipRegion": inclusive voxel box (llf, urb))
        self.enableClipping = False
        self.clipRegion = None
        self.transferFunction = TransFunc1DKeys()
        self.lightPosition = (2.3, 1.5, 1.5, 1.0)
        self.lightAmbient = (0.4, 0.4, 0.4, 1.0)
        self.lightDiffuse = (0.8, 0.8, 0.8, 1.0)
        self.lightSpecular = (0.6, 0.6, 0.6, 1.0)
        self.materialShininess = 60.0
        self.applyLightAttenuation = False
        self.lightAttenuation = (1.0, 0.0, 0.0)
        self.camera = make_camera((0.0, 0.0, 3.0), (0.0, 0.0, 0.0))
        self.brickPoolPlacement = "device"
        self.brickBufferSizeMB = 0
        self.brickUploadBudgetMB = 32
        self.useLevelOfDetail = False
        self.useIterativeRefinement = True
        self.invalidated = False
        self.lastError = ""
        self._device = device
        self._ctx = None
        self._vol = None
        self._vol_src = None
        self._preint = None       # (key, PreIntegrationTable): the cached table
        self._vol_placement = None
        self._last_missed = -1

    # Processor lifecycle ---------------------------------------------------
    def initialize(self):
        self._ctx = Context(self._device)

    def deinitialize(self):
        if self._preint is not None:
            self._preint[1].close()
        self._preint = None
        if self._vol is not None:
            self._vol.close()
        self._vol = None
        if self._ctx is not None:
            self._ctx.close()
        self._ctx = None

    def isReady(self) -> bool:
        """volume + entry/exit ports, as CPURaycaster::isReady (cpuraycaster.cpp:82-84)."""
        return self.volumeInport.hasData() and self.entryPort.isConnected() and self.exitPort.isConnected()

    def _error(self, msg: str):
        self.lastError = msg
        log.error(msg)

    def _fit_tf(self, vol: Volume):
        tf = self.transferFunction
        tf.width = TransferFunction.table_width(vol.dtype)
        if not tf.domain_fitted and tf.domain == (0.0, 1.0):
            lo, hi = vol.minmax()
            s, o = vol.desc.rwm_scale, vol.desc.rwm_offset
            tf.domain = (lo * s + o, hi * s + o)
            tf.domain_fitted = True

    def _preint_table(self, step: float) -> PreIntegrationTable:
        t = self.transferFunction
        res = PreIntegrationTable.resolution(t.width, self.preIntegrationTableSize)
        integral = self.classification == "pre-integrated-approximation"
        key = (step, res, integral, repr(t.keys), t.gamma, tuple(t.threshold))
        if self._preint is None or self._preint[0] != key:
            if self._preint is not None:
                self._preint[1].close()
            src = PreIntegrationTable.bake_source(t.keys, res, t.gamma, t.threshold)
            self._preint = (key, PreIntegrationTable(self._ctx, src, step, integral))
        return self._preint[1]

    def process(self, analytic_entry_exit: bool = False, interacting: bool = False):
        if self._ctx is None:
            self.initialize()
        if not (self.volumeInport.hasData() and (analytic_entry_exit or self.isReady())):
            self._error("not ready: volume and entry/exit points are required")
            return
        if self.compositing not in COMPOSITING or self.shading not in SHADING:
            self._error(f"unsupported compositing/shading: {self.compositing}/{self.shading}")
            return
        if self.classification not in CLASSIFICATION or self.preIntegrationTableSize not in PREINT_TABLE_SIZES:
            self._error(f"unsupported classification: {self.classification}/{self.preIntegrationTableSize}")
            return
        if self.classification == "pre-integrated-gpu":
            self._error("CPU raycaster does not support computing the pre-integration table on the GPU. "
                        "Falling back to CPU.")
            self.classification = "pre-integrated-cpu"
            return
        if not (1 <= int(self.interactionCoarseness) <= 8) or not (0.01 <= self.interactionQuality <= 1.0):
            self._error(f"interaction settings out of range: {self.interactionCoarseness}/{self.interactionQuality}")
            return
        if not (0.01 <= self.samplingRate <= 20.0):
            self._error(f"samplingRate {self.samplingRate} outside [0.01, 20]")
            return
        if self.brickPoolPlacement not in PLACEMENT or not (0 <= self.brickBufferSizeMB) or \
                not (1 <= self.brickUploadBudgetMB <= 1024):
            self._error(f"brick settings out of range: {self.brickPoolPlacement}/{self.brickBufferSizeMB}/"
                        f"{self.brickUploadBudgetMB}")
            return
        vd: VolumeData = self.volumeInport.getData()
        self.invalidated = False
        try:
            placement = PLACEMENT[self.brickPoolPlacement]
            if self._vol is None or self._vol_src is not vd or self._vol_placement != placement:
                if self._vol is not None:
                    self._vol.close()
                self._vol = Volume(self._ctx, vd.voxels, vd.spacing, vd.offset, vd.rwm, placement=placement)
                self._vol_src = vd
                self._vol_placement = placement
            if placement == PLACE_HOST:
                mb = 1 << 20
                self._vol.set_cache_limit(int(self.brickBufferSizeMB) * mb if self.brickBufferSizeMB else 2**62)
                self._vol.set_cache_upload_budget(int(self.brickUploadBudgetMB) * mb)
                self._vol.set_lod(bool(self.useLevelOfDetail))
            self._fit_tf(self._vol)
            t = self.transferFunction
            rgba = TransferFunction.bake(t.keys, t.width, t.gamma, t.threshold)
            tf = TransferFunction(self._ctx, rgba, t.domain)
            if analytic_entry_exit:
                H, W = self.outport.getData().shape[:2] if self.outport.hasData() else (512, 512)
                entry = exit_pts = None
            else:
                entry, exit_pts = self.entryPort.getData(), self.exitPort.getData()
                H, W = entry.shape[:2]
            p = default_params(W, H)
            p.sampling_rate = self.samplingRate
            p.compositing = COMPOSITING[self.compositing]
            p.shading = SHADING[self.shading]
            p.iso_value = self.isoValue
            p.mida_gamma = self.gammaValue
            if self.classification.startswith("pre-integrated"):
                p.classification = CLASSIFY_PREINTEGRATED
                tf.set_preintegration(self._preint_table(sampling_step(self._vol, self.samplingRate)))
            p.light_position[:] = list(self.lightPosition)
            p.light_ambient[:] = list(self.lightAmbient)[:3]
            p.light_diffuse[:] = list(self.lightDiffuse)[:3]
            p.light_specular[:] = list(self.lightSpecular)[:3]
            p.material_shininess = self.materialShininess
            p.apply_attenuation = 1 if self.applyLightAttenuation else 0
            p.light_attenuation[:] = list(self.lightAttenuation)
            p.camera = self.camera
            p.entry_exit_mode = EE_ANALYTIC if analytic_entry_exit else EE_BUFFERS
            if self.enableClipping and self.clipRegion is not None:
                p.enable_clipping = 1
                p.clip_llf[:] = [int(c) for c in self.clipRegion[0]]
                p.clip_urb[:] = [int(c) for c in self.clipRegion[1]]
            coarse = interacting and int(self.interactionCoarseness) > 1
            if interacting:
                p.sampling_rate = self.samplingRate * self.interactionQuality
            if coarse:
                import torch
                c = int(self.interactionCoarseness)
                p.width, p.height = max(1, W // c), max(1, H // c)
                p.entry_exit_mode = EE_ANALYTIC
                small = torch.empty((p.height, p.width, 4), dtype=torch.float32, device=f"cuda:{self._device}")
                _, stats = render(self._ctx, self._vol, tf, p, None, None, OUT_RGBA32F, small)
                full = torch.empty((H, W, 4), dtype=torch.float32, device=f"cuda:{self._device}")
                image_rescale(self._ctx, small, full, OUT_RGBA32F)
                self._ctx.synchronize()
                img = full.cpu().numpy()
            else:
                img, stats = render(self._ctx, self._vol, tf, p, entry, exit_pts, OUT_RGBA32F)
            tf.close()
            self.outport.setData(img)
            self.lastStats = stats
            if placement == PLACE_HOST and self.useIterativeRefinement:
                # another frame helps while the cache is still filling, or
                # while the bricks read without a slot keep changing; a frame
                # that can bring in nothing new ends the refinement
                cached, reachable, missed = self._vol.cache_info()
                nb = int(np.prod(self._vol.brick_minmax()[2]))
                capacity = (int(self.brickBufferSizeMB) << 20) // max(1, self._vol.host_bytes // nb) \
                    if self.brickBufferSizeMB else reachable
                self.invalidated = cached < min(reachable, capacity) or (missed > 0 and missed != self._last_missed)
                self._last_missed = missed
        except VrcError as e:
            self._error(str(e))
