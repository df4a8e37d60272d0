"""Python binding of the CudaRaycaster processor (include/vrc_processor.h,
csrc/processor.cpp): Voreen's CPURaycaster / SingleVolumeRaycaster surface,
implemented in C++ over the C ABI. Attributes map to the processor's
properties by id, as Voreen's Python bindings do; ports hold numpy data that
the processor borrows for the duration of process().

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

import ctypes as C
import logging
from dataclasses import dataclass, field

import numpy as np

from . import _abi, lib, make_camera, make_desc, read_tfi
from ._abi import F32, U8, U16, Camera, RenderStats, TFKey

log = logging.getLogger("voreen.CudaRaycaster")

# property id -> kind, as include/vrc_processor.h lists them
_FLOAT = ("samplingRate", "isoValue", "gammaValue", "interactionQuality", "materialShininess")
_INT = ("preIntegrationTableSize", "interactionCoarseness", "brickBufferSizeMB", "brickUploadBudgetMB")
_BOOL = ("enableClipping", "applyLightAttenuation", "useLevelOfDetail", "useIterativeRefinement")
_STRING = ("compositing", "shading", "gradient", "classification", "brickPoolPlacement")
_FLOATV = {"lightPosition": 4, "lightAmbient": 4, "lightDiffuse": 4, "lightSpecular": 4, "lightAttenuation": 3}
_NP_DTYPE = {np.dtype(np.uint8): U8, np.dtype(np.uint16): U16, np.dtype(np.float32): F32}


@dataclass
class VolumeData:
    """What a VolumePort carries: voxels (Z, Y, X) plus the metadata the
    march uses (spacing, offset, real-world mapping)."""
    voxels: np.ndarray
    spacing: tuple = (1.0, 1.0, 1.0)
    offset: tuple = (0.0, 0.0, 0.0)
    rwm: tuple = (1.0, 0.0)


class Port:
    """A processor port: its id and the data it currently holds."""

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
    """The transferFunction property: keys as (intensity, colour) or
    (intensity, colourL, colourR), domain, gamma, thresholds, and the table
    width / domain fitting state process() maintains."""
    keys: list = field(default_factory=lambda: [(0.0, (0, 0, 0, 0)), (1.0, (255, 255, 255, 255))])
    domain: tuple = (0.0, 1.0)
    gamma: float = 1.0
    threshold: tuple = (0.0, 1.0)
    width: int = 256
    domain_fitted: bool = False


def _id(name: str) -> bytes:
    return name.encode()


class CudaRaycaster:
    """The C++ CudaRaycaster processor (include/vrc_processor.h) with its
    ports as attributes and its properties readable and writable by id."""
    className = "CudaRaycaster"
    category = "Raycasting"

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        st = lib().vrcp_create(device, C.byref(h))
        if st != _abi.VRC_OK:
            raise RuntimeError(f"vrcp_create: {st}")
        object.__setattr__(self, "_h", h)
        object.__setattr__(self, "volumeInport", Port("volumehandle.volumehandle"))
        object.__setattr__(self, "entryPort", Port("image.entrypoints"))
        object.__setattr__(self, "exitPort", Port("image.exitpoints"))
        object.__setattr__(self, "outport", Port("image.output"))
        object.__setattr__(self, "transferFunction", TransFunc1DKeys())
        object.__setattr__(self, "camera", make_camera((0.0, 0.0, 3.0), (0.0, 0.0, 0.0)))
        object.__setattr__(self, "clipRegion", None)
        object.__setattr__(self, "lastStats", None)
        object.__setattr__(self, "_vol_src", None)
        object.__setattr__(self, "_borrowed", ())

    # properties by id ------------------------------------------------------
    def __getattr__(self, name):
        L, h = lib(), object.__getattribute__(self, "_h")
        if name in _FLOAT:
            v = C.c_float()
            L.vrcp_get_float(h, _id(name), C.byref(v))
            return v.value
        if name in _INT or name in _BOOL:
            v = C.c_int()
            L.vrcp_get_int(h, _id(name), C.byref(v))
            return bool(v.value) if name in _BOOL else v.value
        if name in _STRING:
            buf = C.create_string_buffer(256)
            L.vrcp_get_string(h, _id(name), buf, 256)
            return buf.value.decode()
        if name in _FLOATV:
            n = _FLOATV[name]
            v = (C.c_float * n)()
            L.vrcp_get_floatv(h, _id(name), v, n)
            return tuple(float(x) for x in v)
        if name == "lastError":
            return (L.vrcp_last_error(h) or b"").decode()
        if name == "invalidated":
            return bool(L.vrcp_invalidated(h))
        raise AttributeError(name)

    def __setattr__(self, name, value):
        L, h = lib(), self._h
        if name in _FLOAT:
            L.vrcp_set_float(h, _id(name), float(value))
        elif name in _INT or name in _BOOL:
            L.vrcp_set_int(h, _id(name), int(value))
        elif name in _STRING:
            L.vrcp_set_string(h, _id(name), str(value).encode())
        elif name in _FLOATV:
            n = _FLOATV[name]
            v = [float(x) for x in value][:n]
            v += [1.0] * (n - len(v))
            L.vrcp_set_floatv(h, _id(name), (C.c_float * n)(*v), n)
        else:
            object.__setattr__(self, name, value)

    # Processor lifecycle ---------------------------------------------------
    def initialize(self):
        lib().vrcp_initialize(self._h)

    def deinitialize(self):
        lib().vrcp_deinitialize(self._h)

    def close(self):
        if self._h:
            lib().vrcp_destroy(self._h)
            object.__setattr__(self, "_h", C.c_void_p())

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load_transfer_function(self, path: str):
        """Loads a Voreen .tfi file into transferFunction (keys, gamma,
        thresholds and the file's domain, which process() keeps)."""
        st = lib().vrcp_load_tf(self._h, path.encode())
        if st != _abi.VRC_OK:
            raise RuntimeError(f"vrcp_load_tf({path}): {_abi.STATUS_NAMES.get(st, st)}")
        t = read_tfi(path)
        self.transferFunction.keys = [(k[0], k[1], k[2]) for k in t["keys"]]
        self.transferFunction.gamma = t["gamma"]
        self.transferFunction.threshold = t["threshold"]
        self.transferFunction.domain = t["domain"]
        self.transferFunction.domain_fitted = True

    def isReady(self) -> bool:
        """volume + entry/exit ports, as CPURaycaster::isReady (cpuraycaster.cpp:82-84)."""
        return self.volumeInport.hasData() and self.entryPort.isConnected() and self.exitPort.isConnected()

    def _push(self):
        """Hands the port data and the compound properties to the processor."""
        L, h = lib(), self._h
        borrowed = []
        vd = self.volumeInport.getData()
        if vd is None:
            if self._vol_src is not None:
                L.vrcp_set_volume(h, None, None)
            object.__setattr__(self, "_vol_src", None)
        elif vd is not self._vol_src:
            vox = np.ascontiguousarray(vd.voxels)
            desc = make_desc(_NP_DTYPE[vox.dtype], vox.shape[::-1], vd.spacing, vd.offset, vd.rwm)
            L.vrcp_set_volume(h, C.byref(desc), vox.ctypes.data_as(C.c_void_p))
            object.__setattr__(self, "_vol_src", vd)
            object.__setattr__(self, "_vol_array", vox)
        e, x = self.entryPort.getData(), self.exitPort.getData()
        if e is not None and x is not None:
            e = np.ascontiguousarray(e, dtype=np.float32)
            x = np.ascontiguousarray(x, dtype=np.float32)
            borrowed += [e, x]
            L.vrcp_set_entry_exit(h, e.ctypes.data_as(C.c_void_p), x.ctypes.data_as(C.c_void_p), e.shape[1],
                                  e.shape[0])
        else:
            L.vrcp_set_entry_exit(h, None, None, 0, 0)
        out = self.outport.getData()
        if out is not None:
            L.vrcp_set_output_size(h, out.shape[1], out.shape[0])
        t = self.transferFunction
        keys = (TFKey * max(1, len(t.keys)))()
        for i, k in enumerate(t.keys):
            keys[i].intensity = float(k[0])
            keys[i].color_l[:] = [int(v) for v in k[1]]
            keys[i].color_r[:] = [int(v) for v in (k[2] if len(k) > 2 else k[1])]
        L.vrcp_set_tf_keys(h, keys, len(t.keys), float(t.gamma), float(t.threshold[0]), float(t.threshold[1]))
        L.vrcp_set_tf_domain(h, float(t.domain[0]), float(t.domain[1]), 1 if t.domain_fitted else 0, int(t.width))
        cam = self.camera
        if not isinstance(cam, Camera):
            cam = make_camera(cam.position, cam.focus)
        L.vrcp_set_camera(h, C.byref(cam))
        if self.clipRegion is None:
            L.vrcp_set_intv(h, b"clipRegion", None, 0)
        else:
            v = [int(c) for c in self.clipRegion[0]] + [int(c) for c in self.clipRegion[1]]
            L.vrcp_set_intv(h, b"clipRegion", (C.c_int * 6)(*v), 6)
        object.__setattr__(self, "_borrowed", tuple(borrowed))

    def _pull(self):
        L, h = lib(), self._h
        w, lo, hi, fitted = C.c_int(), C.c_float(), C.c_float(), C.c_int()
        L.vrcp_get_tf(h, C.byref(w), C.byref(lo), C.byref(hi), C.byref(fitted))
        t = self.transferFunction
        t.width, t.domain, t.domain_fitted = w.value, (lo.value, hi.value), bool(fitted.value)
        ptr, W, H = C.POINTER(C.c_float)(), C.c_int(), C.c_int()
        if L.vrcp_output(h, C.byref(ptr), C.byref(W), C.byref(H)):
            img = np.ctypeslib.as_array(ptr, shape=(H.value, W.value, 4)).copy()
            self.outport.setData(img)
            st = RenderStats()
            L.vrcp_last_stats(h, C.byref(st))
            object.__setattr__(self, "lastStats", st)

    def process(self, analytic_entry_exit: bool = False, interacting: bool = False):
        """One frame into outport (CPURaycaster::process; interaction mode as
        SingleVolumeRaycaster's). On failure: lastError, no new output."""
        self._push()
        lib().vrcp_process(self._h, 1 if analytic_entry_exit else 0, 1 if interacting else 0)
        self._pull()
        object.__setattr__(self, "_borrowed", ())
        err = self.lastError
        if err:
            log.error(err)
