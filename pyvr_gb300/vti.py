"""VTK XML ImageData (``.vti``) reader and writer without the vtk package.

``load_vtk_volume`` has the behaviour of pyvr/dataloaders/vtk_loader.py:15-146:

- it reads one single-component point-data array;
- it reshapes the array to (nz, ny, nx), because VTK stores x fastest;
- it normalises to [0, 1] in float32 (a constant volume becomes zeros);
- it sizes the bounds from the physical extent dims × spacing, longest axis to [-1, 1],
  centred at 0;
- it names the volume ``file(Scalars)`` and computes the normals.

The file format is parsed here directly:

- the XML structure of VTKFile / ImageData / Piece / PointData / DataArray;
- DataArray payloads in ``ascii``, inline ``binary`` (base64) and ``appended`` (raw or
  base64) form;
- UInt32 or UInt64 size headers, little- or big-endian data;
- uncompressed or block-compressed payloads (vtkZLibDataCompressor, vtkLZMADataCompressor).

A compressed payload starts with a header [number of blocks, uncompressed block size,
size of the last partial block (0 if full), compressed size of each block], followed by
the compressed blocks. In base64 form the header and the blocks are encoded as two separate
base64 runs. An uncompressed payload starts with one header integer, the byte count.
"""

from __future__ import annotations

import base64
import lzma
import xml.etree.ElementTree as ET
import zlib
from pathlib import Path
from typing import Dict, Optional, Tuple, Union

import numpy as np

from .volume import Volume

_TYPES = {"Int8": "i1", "UInt8": "u1", "Int16": "i2", "UInt16": "u2", "Int32": "i4", "UInt32": "u4",
          "Int64": "i8", "UInt64": "u8", "Float32": "f4", "Float64": "f8"}
_DECOMPRESS = {"vtkZLibDataCompressor": zlib.decompress, "vtkLZMADataCompressor": lzma.decompress}


class _Payload:
    """Decoder of one DataArray's bytes."""

    def __init__(self, root: ET.Element, raw_appended: Optional[bytes]):
        self.order = "<" if root.get("byte_order", "LittleEndian") == "LittleEndian" else ">"
        htype = root.get("header_type", "UInt32")
        if htype not in ("UInt32", "UInt64"):
            raise ValueError(f"unsupported header_type {htype!r}")
        self.hdt = np.dtype(self.order + ("u4" if htype == "UInt32" else "u8"))
        comp = root.get("compressor")
        if comp and comp not in _DECOMPRESS:
            raise ValueError(f"unsupported compressor {comp!r}")
        self.decompress = _DECOMPRESS.get(comp) if comp else None
        self.appended = raw_appended
        app = root.find("AppendedData")
        self.app_encoding = app.get("encoding", "raw") if app is not None else None

    def _ints(self, b: bytes, n: int) -> np.ndarray:
        return np.frombuffer(b[:n * self.hdt.itemsize], dtype=self.hdt).astype(np.int64)

    def _from_b64_stream(self, text: bytes) -> bytes:
        """Header and data encoded as separate base64 runs (or together: detected)."""
        hs = self.hdt.itemsize
        if self.decompress is None:
            hlen = 4 * ((hs + 2) // 3)
            head = base64.b64decode(text[:hlen])
            if text[hlen - 1:hlen] == b"=" or len(head) == hs:  # separate runs
                nbytes = int(self._ints(head, 1)[0])
                return base64.b64decode(text[hlen:hlen + 4 * ((nbytes + 2) // 3)])[:nbytes]
            allb = base64.b64decode(text)  # header and data in one run
            nbytes = int(self._ints(allb, 1)[0])
            return allb[hs:hs + nbytes]
        first = base64.b64decode(text[:4 * ((hs + 2) // 3)])
        nblocks = int(self._ints(first, 1)[0])
        hbytes = (3 + nblocks) * hs
        hlen = 4 * ((hbytes + 2) // 3)
        head = base64.b64decode(text[:hlen])
        sizes = self._ints(head, 3 + nblocks)
        total = int(sizes[3:].sum())
        body = base64.b64decode(text[hlen:hlen + 4 * ((total + 2) // 3)])[:total]
        return self._blocks(sizes, body)

    def _blocks(self, sizes: np.ndarray, body: bytes) -> bytes:
        nblocks, bsize, last = int(sizes[0]), int(sizes[1]), int(sizes[2])
        out, off = [], 0
        for k in range(nblocks):
            c = int(sizes[3 + k])
            block = self.decompress(body[off:off + c])
            want = last if (k == nblocks - 1 and last) else bsize
            if len(block) != want:
                raise ValueError("corrupt compressed block")
            out.append(block)
            off += c
        return b"".join(out)

    def _from_raw(self, raw: bytes) -> bytes:
        hs = self.hdt.itemsize
        if self.decompress is None:
            nbytes = int(self._ints(raw, 1)[0])
            return raw[hs:hs + nbytes]
        nblocks = int(self._ints(raw, 1)[0])
        sizes = self._ints(raw, 3 + nblocks)
        start = (3 + nblocks) * hs
        return self._blocks(sizes, raw[start:start + int(sizes[3:].sum())])

    def read(self, arr: ET.Element) -> np.ndarray:
        t = arr.get("type")
        if t not in _TYPES:
            raise ValueError(f"unsupported DataArray type {t!r}")
        dt = np.dtype(self.order + _TYPES[t])
        fmt = arr.get("format", "ascii")
        if fmt == "ascii":
            return np.array((arr.text or "").split(), dtype=dt.newbyteorder("="))
        if fmt == "binary":
            data = self._from_b64_stream("".join((arr.text or "").split()).encode())
        elif fmt == "appended":
            if self.appended is None:
                raise ValueError("appended DataArray without AppendedData")
            off = int(arr.get("offset", "0"))
            if self.app_encoding == "base64":
                data = self._from_b64_stream(self.appended[off:])
            else:
                data = self._from_raw(self.appended[off:])
        else:
            raise ValueError(f"unsupported DataArray format {fmt!r}")
        return np.frombuffer(data, dtype=dt).astype(dt.newbyteorder("="))


def _split_appended(blob: bytes) -> Tuple[bytes, Optional[bytes]]:
    """XML text with the appended payload removed, and the payload (the bytes
    after the '_' marker up to the closing tag)."""
    start = blob.find(b"<AppendedData")
    if start < 0:
        return blob, None
    mark = blob.find(b"_", blob.find(b">", start))
    end = blob.rfind(b"</AppendedData>")
    if mark < 0 or end < 0:
        raise ValueError("malformed AppendedData section")
    payload = blob[mark + 1:end]
    head = blob[:blob.find(b">", start) + 1]
    return head + b"</AppendedData></VTKFile>", payload


def read_vti(file_path: Union[str, Path]) -> Dict:
    """The ImageData of a ``.vti`` file: dims (nx, ny, nz), spacing, origin,
    its point-data arrays {name: (DataArray element, components)}, and the
    payload decoder (``img["_payload"].read(element)`` gives the flat array)."""
    with open(file_path, "rb") as f:
        blob = f.read()
    xml_text, appended = _split_appended(blob)
    root = ET.fromstring(xml_text)
    if root.tag != "VTKFile" or root.get("type") != "ImageData":
        raise ValueError("not a VTK ImageData file")
    img = root.find("ImageData")
    if img is None:
        raise ValueError("no ImageData element")
    ext = [int(v) for v in img.get("WholeExtent").split()]
    dims = (ext[1] - ext[0] + 1, ext[3] - ext[2] + 1, ext[5] - ext[4] + 1)
    spacing = tuple(float(v) for v in img.get("Spacing", "1 1 1").split())
    origin = tuple(float(v) for v in img.get("Origin", "0 0 0").split())
    pieces = img.findall("Piece")
    if len(pieces) != 1:
        raise ValueError(f"{len(pieces)} pieces; one piece is supported")
    if appended is not None and root.find("AppendedData").get("encoding", "raw") == "base64":
        appended = b"".join(appended.split())  # raw payloads are used as they are
    payload = _Payload(root, appended)
    arrays = {}
    pd = pieces[0].find("PointData")
    for arr in (pd.findall("DataArray") if pd is not None else []):
        arrays[arr.get("Name")] = (arr, int(arr.get("NumberOfComponents", "1")))
    return {"dims": dims, "spacing": spacing, "origin": origin, "arrays": arrays, "_payload": payload}


def load_vtk_volume(file_path: Union[str, Path], scalars_name: str = "Scalars_",
                    compute_normals: bool = True) -> Volume:
    """A ``.vti`` file as a Volume, as pyvr/dataloaders/vtk_loader.py:15-146
    builds it (normalised float32 data, aspect-preserving bounds in [-1, 1],
    name ``file(Scalars)``, normals computed).  compute_normals=False
    (extension) leaves the normals to the GPU layout (``DeviceVolume(...,
    normals="device")``), which gives the same normals."""
    file_path = Path(file_path)
    if not file_path.exists():
        raise FileNotFoundError(f"VTK file not found: {file_path}")
    img = read_vti(file_path)
    dims, spacing = img["dims"], img["spacing"]
    if any(d <= 0 for d in dims):
        raise ValueError(f"Invalid dimensions: {dims}")
    if any(s <= 0 for s in spacing):
        raise ValueError(f"Invalid spacing (must be positive): {spacing}")
    if scalars_name not in img["arrays"]:
        raise ValueError(f"Scalar array '{scalars_name}' not found in {file_path}. "
                         f"Available arrays: {list(img['arrays'])}")
    elem, comps = img["arrays"][scalars_name]
    if comps != 1:
        raise ValueError(f"Multi-component scalars not supported. Array '{scalars_name}' has "
                         f"{comps} components, expected 1.")
    flat = img["_payload"].read(elem)
    n = dims[0] * dims[1] * dims[2]
    if flat.size != n:
        raise ValueError(f"array '{scalars_name}' has {flat.size} values, expected {n}")
    data = flat.reshape((dims[2], dims[1], dims[0])).astype(np.float32)
    lo, hi = data.min(), data.max()
    if hi - lo < 1e-9:
        norm = np.zeros_like(data)
    else:
        norm = (data - lo) / (hi - lo)
    phys = np.array([dims[0] * spacing[0], dims[1] * spacing[1], dims[2] * spacing[2]], dtype=np.float32)
    scale = 2.0 / np.max(phys)
    half = phys * scale / 2.0
    vol = Volume(data=norm, normals=None, min_bounds=-half, max_bounds=+half,
                 name=f"{file_path.name}({scalars_name})")
    if compute_normals:
        vol.compute_normals()
    return vol


def write_vti(file_path: Union[str, Path], data: np.ndarray, spacing=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0),
              name: str = "Scalars_", fmt: str = "appended", encoding: str = "raw", compress: bool = False,
              header_type: str = "UInt32", block_size: int = 1 << 15) -> None:
    """Write a (nz, ny, nx) array as single-component point data.
    fmt: 'ascii', 'binary' (inline base64) or 'appended' (encoding 'raw' or
    'base64'); compress: zlib blocks of block_size bytes."""
    data = np.ascontiguousarray(data)
    inv = {v: k for k, v in _TYPES.items()}
    tname = inv[data.dtype.newbyteorder("=").str[1:]]
    nz, ny, nx = data.shape
    hdt = np.dtype("<u4" if header_type == "UInt32" else "<u8")
    raw = data.astype(data.dtype.newbyteorder("<")).tobytes()
    if compress:
        blocks = [raw[i:i + block_size] for i in range(0, len(raw), block_size)] or [b""]
        comp = [zlib.compress(b) for b in blocks]
        last = len(blocks[-1]) if len(blocks[-1]) != block_size else 0
        head = np.array([len(blocks), block_size, last] + [len(c) for c in comp], dtype=hdt).tobytes()
        body = b"".join(comp)
    else:
        head = np.array([len(raw)], dtype=hdt).tobytes()
        body = raw
    attrs = (f'type="ImageData" version="1.0" byte_order="LittleEndian" header_type="{header_type}"'
             + (' compressor="vtkZLibDataCompressor"' if compress else ""))
    ext = f"0 {nx - 1} 0 {ny - 1} 0 {nz - 1}"
    if fmt == "ascii":
        arr = (f'<DataArray type="{tname}" Name="{name}" format="ascii">'
               + " ".join(repr(v) for v in data.ravel().tolist()) + "</DataArray>")
        tail = b""
    elif fmt == "binary":
        enc = (base64.b64encode(head) + base64.b64encode(body)).decode()
        arr = f'<DataArray type="{tname}" Name="{name}" format="binary">{enc}</DataArray>'
        tail = b""
    else:
        arr = f'<DataArray type="{tname}" Name="{name}" format="appended" offset="0"/>'
        if encoding == "base64":
            tail = (b'<AppendedData encoding="base64">_' + base64.b64encode(head) + base64.b64encode(body)
                    + b"</AppendedData>")
        else:
            tail = b'<AppendedData encoding="raw">_' + head + body + b"</AppendedData>"
    xml = (f'<?xml version="1.0"?>\n<VTKFile {attrs}>\n'
           f'<ImageData WholeExtent="{ext}" Origin="{" ".join(map(str, origin))}" '
           f'Spacing="{" ".join(map(str, spacing))}">\n<Piece Extent="{ext}">\n'
           f'<PointData Scalars="{name}">{arr}</PointData>\n<CellData></CellData>\n</Piece>\n</ImageData>\n')
    with open(file_path, "wb") as f:
        f.write(xml.encode() + tail + b"\n</VTKFile>\n")
