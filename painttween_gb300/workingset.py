"""Working sets: the reference's XML description of a synthesis job, loaded
without Qt (GUI/nlSynthesizer.cpp:99-160).

    <doc>
      <styles>
        <style frame="12">            (frame: the style is the key of that frame)
          <styleInput path="..."/> <styleOutput path="..."/>
          <styleDistanceTransform path="..."/> <styleOrientation path="..."/>
          <styleObjectIDs path="..."/>
        </style> ...
      </styles>
      <params> <levels value="5"/> <coherenceWeight value="0"/> ...
               <offsetsHistogramSlope value0="..." value1="..."/> ... </params>
      <anim>
        <unit name="..."/> <shot name="..."/> <shotDir path="..."/>
        <workingDir path="..."/> <fileAccess checkFarm="0"/>
        <elements inputElem="rgba" orientationElem="..." distTransElem="..."
                  scaleElem="..." idMergedElem="..." velBElem="..." velFElem="..."
                  ribbonBElem="vel_b_[NN]" ribbonFElem="vel_f_[NN]"/>
      </anim>
    </doc>

Paths are relative to the XML file.  Style images are read by the channel
names of their layer (GUI/nlStyles.cpp:33-40: "style_input.red" ...), input
elements from `<shotDir>/<shot>.<element>.<frame>.exr` (GUI/nlShot.cpp:
139-160; with checkFarm `<shotDir>/<element>/<shot>.<element>.<frame>.exr`)
by their layer's channels (GUI/nlInputElements.cpp:30-42); the "rgba" input
layer is the file's R, G, B, A.  As with OpenEXR's reader, a channel missing
from a file reads zero; a missing input element takes the reference's
default (zero, scale 1).  Object IDs become r + 255 g + 255^2 b of the
rounded 8-bit colour (imageIO.cpp:299-320).  Parameters map onto pt_params
as SynthesisProcessor::updateParameters does (synthesisProcessor.cpp:
175-262): `maxLevel` is the final level, `synthesisScheme` the scheme.
"""
import os
import xml.etree.ElementTree as ET

import numpy as np

from . import _abi, exr

_STYLE_LAYERS = (("base", "styleInput", "style_input", ("red", "green", "blue", "alpha")),
                 ("output", "styleOutput", "style_output", ("red", "green", "blue", "alpha")),
                 ("dist_trans", "styleDistanceTransform", "dist_trans", ("length",)),
                 ("orient_tensor", "styleOrientation", "orientation", ("Ix2", "IxIy", "Iy2")),
                 ("object_ids", "styleObjectIDs", "id", ("red", "green", "blue")))
_INPUT_LAYERS = (("rgba", "inputElem", "rgba", ("R", "G", "B", "A")),
                 ("orient_tensor", "orientationElem", "orientation", ("Ix2", "IxIy", "Iy2")),
                 ("dist_trans", "distTransElem", "dist_trans", ("length",)),
                 ("scale", "scaleElem", "scale", ("x", "y")),
                 ("object_ids", "idMergedElem", "id", ("red", "green", "blue")),
                 ("vel_bwd", "velBElem", "vel_b_1", ("x", "y")),
                 ("vel_fwd", "velFElem", "vel_f_1", ("x", "y")))

_FLOATS = {"coherenceWeight": "coherenceWeight", "hysteresisWeight": "hysteresisWeight",
           "maxDistortion": "maxDistortion", "inputAnalogyWeight": "inputAnalogyWeight",
           "canvasOutputWeight": "canvasOutputWeight", "distanceTransformWeight": "distTransWeight",
           "timeDerivativeInputWeight": "timeDerivativeInputWeight",
           "timeDerivativeOutputWeight": "timeDerivativeOutputWeight",
           "temporalCoherenceWeight": "temporalCoherenceWeight", "styleObjectIdWeight": "styleObjIdWeight",
           "advectionJitter": "advectionJitter", "lumShiftWeight": "lumShiftWeight",
           "alphaChannelWeight": "alphaWeight", "residualWindowScaleU": "residualWindowScaleU",
           "residualWindowScaleV": "residualWindowScaleV"}
_BOOLS = {"orientationEnabled": "orientationEnabled", "keyFrameInterpolation": "interpolateKeyFrame",
          "guidedInterpolation": "useGuide", "lumShiftEnabled": "lumShiftEnable",
          "transparencyAllowed": "transparencyOk"}
_INTS = {"iterations": "iterations", "levels": "levels", "maxLevel": "finalLevel",
         "scatterSamplesCount": "scatterSamplesCount", "fixupPasses": "fixupPasses",
         "residualWindowSize": "residualWindowSize", "colorspace": "colorspace", "synthesisScheme": "scheme"}


class WorkingSetError(ValueError):
    pass


def _channels(img, layer, names):
    ch = img["channels"]
    h, w = img["height"], img["width"]
    out = np.zeros((h, w, len(names)), np.float32)
    for i, n in enumerate(names):
        key = n if layer == "rgba" else "%s.%s" % (layer, n)
        if key in ch:
            out[..., i] = ch[key].astype(np.float32)
    if layer == "rgba" and "A" not in ch:
        out[..., 3] = 1.0
    return out


def _ids(rgb):
    r, g, b = (np.floor(rgb[..., i] * np.float32(255) + 0.5).astype(np.int64) for i in range(3))
    return (r + g * 255 + b * 255 * 255).astype(np.int32)


def _image(path, key, layer, names):
    a = _channels(exr.read(path), layer, names)
    if key == "object_ids":
        return _ids(a)
    return a[..., 0] if a.shape[-1] == 1 else a


class WorkingSet:
    """A parsed working set: `params` (pt_params), `styles` (dicts for
    Synthesizer.set_style), `keyframes` (frame of each keyed style, in style
    order), `first_frame`, `last_frame`, and `frame(f)` to read one frame's
    inputs (a dict for Synthesizer.set_frame_dict)."""

    def __init__(self, path):
        self.path = os.path.abspath(path)
        root_dir = os.path.dirname(self.path)
        doc = ET.parse(self.path).getroot()
        styles = doc.find("styles")
        if styles is None:
            raise WorkingSetError("no <styles> element")
        self.styles, self.keyframes = [], []
        for st in styles:
            if "frame" in st.attrib:
                self.keyframes.append(int(st.attrib["frame"]))
            d = {}
            for key, xml, layer, names in _STYLE_LAYERS:
                el = st.find(xml)
                if el is not None and "path" in el.attrib:
                    d[key] = _image(os.path.normpath(os.path.join(root_dir, el.attrib["path"])), key, layer, names)
            if "base" not in d or "output" not in d:
                raise WorkingSetError("a style needs styleInput and styleOutput")
            self.styles.append(d)
        self.params = _abi.default_params()
        p = self.params
        p.residualWindowSize = 4  # NLParameters::getTsDefaultParams
        pe = doc.find("params")
        self.first_frame = self.last_frame = 0
        if pe is not None:
            for el in pe:
                name, v = el.tag, el.attrib.get("value")
                if name in ("offsetsHistogramSlope", "offsetsHistogramThreshold"):
                    arr = p.offsetsHistogramSlope if name.endswith("Slope") else p.offsetsHistogramThreshold
                    for i in range(min(len(self.styles), _abi.PT_MAX_STYLES)):
                        if "value%d" % i in el.attrib:
                            arr[i] = float(el.attrib["value%d" % i])
                elif name in _FLOATS and v is not None:
                    setattr(p, _FLOATS[name], float(v))
                elif name in _BOOLS and v is not None:
                    setattr(p, _BOOLS[name], 1 if int(v) == 1 else 0)
                elif name in _INTS and v is not None:
                    setattr(p, _INTS[name], int(v))
                elif name == "firstFrame" and v is not None:
                    self.first_frame = int(v)
                elif name == "lastFrame" and v is not None:
                    self.last_frame = int(v)
        p.numStyles = len(self.styles)
        anim = doc.find("anim")
        if anim is None:
            raise WorkingSetError("no <anim> element")

        def attr(tag, name):
            el = anim.find(tag)
            if el is None or name not in el.attrib:
                raise WorkingSetError("<anim> lacks %s %s" % (tag, name))
            return el.attrib[name]

        self.shot = attr("shot", "name")
        self.shot_dir = os.path.normpath(os.path.join(root_dir, attr("shotDir", "path")))
        self.working_dir = os.path.normpath(os.path.join(root_dir, attr("workingDir", "path")))
        fa = anim.find("fileAccess")
        farm = self.farm = fa is not None and fa.attrib.get("checkFarm", "0").strip() == "1"
        el = anim.find("elements")
        self.elements = {}
        for key, xml, layer, names in _INPUT_LAYERS:
            name = el.attrib.get(xml, "").strip(".") if el is not None else ""
            if name:
                base = os.path.join(self.shot_dir, name, self.shot) if farm else os.path.join(self.shot_dir, self.shot)
                self.elements[key] = (base + "." + name + ".%d.exr", layer, names)
        if "rgba" not in self.elements:
            raise WorkingSetError("no input element (inputElem)")
        # ribbon elements (GUI/nlShot.cpp:162-190): "[..]" in the name is the
        # two-digit step; without checkFarm the files are named relative to
        # the working directory of the process, as in the reference
        self.ribbon_elements = {}
        for key, xml in (("vel_bwd", "ribbonBElem"), ("vel_fwd", "ribbonFElem")):
            name = el.attrib.get(xml, "").strip(".") if el is not None else ""
            if name:
                self.ribbon_elements[key] = name

    def _ribbon_path(self, key, step, frame):
        import re
        elem = re.sub(r"\[.*\]", "%02d" % step, self.ribbon_elements[key])
        if self.farm:
            return os.path.join(self.shot_dir, elem, self.shot + "." + elem) + ".%d.exr" % frame
        return elem + ".%d.exr" % frame

    def ribbon_steps(self, first, last):
        """Steps 1, 2, 4 ... whose ribbon files exist for every frame, up to
        the first missing one (at most 512)."""
        steps = []
        if len(self.ribbon_elements) < 2:
            return steps
        for i in range(10):
            st = 1 << i
            if not all(os.path.exists(self._ribbon_path(k, st, f)) for k in ("vel_bwd", "vel_fwd")
                       for f in range(first, last + 1)):
                break
            steps.append(st)
        return steps

    def ribbons(self, frame, step):
        """(vel_fwd, vel_bwd) of one frame and step; the layer is vel_f_<step>
        / vel_b_<step>."""
        out = []
        for key, layer in (("vel_fwd", "vel_f_%d" % step), ("vel_bwd", "vel_b_%d" % step)):
            out.append(_image(self._ribbon_path(key, step, frame), key, layer, ("x", "y")))
        return tuple(out)

    def frame_path(self, key, frame):
        return self.elements[key][0] % frame

    def frame(self, f):
        """One frame's inputs; absent elements take the reference's defaults."""
        d = {}
        for key, (pattern, layer, names) in self.elements.items():
            path = pattern % f
            if os.path.exists(path):
                d[key] = _image(path, key, layer, names)
        h, w = d["rgba"].shape[:2]
        d.setdefault("orient_tensor", np.zeros((h, w, 3), np.float32))
        d.setdefault("dist_trans", np.zeros((h, w), np.float32))
        d.setdefault("object_ids", np.zeros((h, w), np.int32))
        d.setdefault("scale", np.ones((h, w, 2), np.float32))
        d.setdefault("vel_fwd", np.zeros((h, w, 2), np.float32))
        d.setdefault("vel_bwd", np.zeros((h, w, 2), np.float32))
        d["w"], d["h"] = w, h
        return d

    def setup(self, synth, first=None, last=None):
        """Feeds a Synthesizer: context sizes, parameters, styles, keyframes
        and the frames first..last (default: the working set's range, widened
        to the keys next to it when keyframe interpolation is on)."""
        first = self.first_frame if first is None else first
        last = self.last_frame if last is None else last
        fr0 = self.frame(first)
        sh, sw = self.styles[0]["base"].shape[:2]
        synth.setup(self.params, fr0["w"], fr0["h"], sw, sh, len(self.styles))
        for i, s in enumerate(self.styles):
            synth.set_style(i, s["base"], s["output"], s.get("orient_tensor"), s.get("dist_trans"),
                            s.get("object_ids"))
        lo, hi = first, last
        if self.params.interpolateKeyFrame and self.keyframes:
            synth.set_keyframes(self.keyframes)
            lo = min([first] + [k for k in self.keyframes if k < first][-1:])
            hi = max([last] + [k for k in self.keyframes if k > last][:1])
        for f in range(lo, hi + 1):
            synth.set_frame_dict(f, fr0 if f == first else self.frame(f))
        for st in self.ribbon_steps(lo, hi)[1:]:  # step 1 is the frames' own velocities
            for f in range(lo, hi + 1):
                synth.set_frame_ribbons(f, st, *self.ribbons(f, st))
        return first, last


def load(path):
    return WorkingSet(path)
