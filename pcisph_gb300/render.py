"""Headless frames of a simulation: the reference's particle rendering (pcisph_render) written as PNG.

Replaces the window, the OpenGL draw and the frame recording of the reference's main loop
(PCISPH/src/main.cpp:174-220): reference_camera() is its camera, record() steps a context and writes a
frame every `interval` seconds of simulated time like the recording branch (main.cpp:191-220), and
write_png() stores RGB8 images (the reference used stbi_write_png).
"""
import ctypes as C
import math
import os
import struct
import zlib

import numpy as np

from ._lib import Camera, check, load


def reference_camera(distance=9.0, angle=0.0, fov_x_degrees=60.0):
    """main.cpp:174-179: eye at distance * (sin a, 0.2, cos a), looking at the origin, +y up."""
    c = Camera()
    c.eye[:] = [distance * math.sin(angle), distance * 0.2, distance * math.cos(angle)]
    c.target[:] = [0.0, 0.0, 0.0]
    c.up[:] = [0.0, 1.0, 0.0]
    c.fov_x_degrees = fov_x_degrees
    return c


def camera(eye, target, up=(0.0, 1.0, 0.0), fov_x_degrees=60.0):
    c = Camera()
    c.eye[:], c.target[:], c.up[:] = [float(v) for v in eye], [float(v) for v in target], [float(v) for v in up]
    c.fov_x_degrees = fov_x_degrees
    return c


def render(fluid, cam, width=640, height=480):
    """The context's fluid as an (height, width, 3) uint8 image."""
    out = np.empty((height, width, 3), np.uint8)
    check(load().pcisph_render_fluid(fluid._h, C.byref(cam), int(width), int(height),
                                     C.c_void_p(out.ctypes.data), out.nbytes))
    return out


def write_png(path, rgb):
    """An (h, w, 3) uint8 array as an 8-bit RGB PNG (zlib stream, no filtering)."""
    rgb = np.ascontiguousarray(rgb, np.uint8)
    h, w, _ = rgb.shape
    raw = b"".join(b"\x00" + rgb[y].tobytes() for y in range(h))

    def chunk(kind, data):
        body = kind + data
        return struct.pack(">I", len(data)) + body + struct.pack(">I", zlib.crc32(body) & 0xFFFFFFFF)
    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0))
    png += chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(png)


def read_png(path):
    """Inverse of write_png (unfiltered 8-bit RGB PNGs only)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        if kind == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 3 * w)
    return raw[:, 1:].reshape(h, w, 3).copy()


def record(fluid, duration, interval, out_dir, cam=None, width=640, height=480):
    """Step `fluid` for `duration` seconds of simulated time, writing out_dir/frame_<k>.png every
    `interval` seconds (main.cpp:191-220); returns the frame paths."""
    cam = cam or reference_camera()
    os.makedirs(out_dir, exist_ok=True)
    dt = fluid.get_params().delta_t
    t, last, paths = 0.0, 0.0, []
    while t < duration:
        fluid.update()
        t += dt
        if t - last >= interval:
            path = os.path.join(out_dir, f"frame_{len(paths)}.png")
            write_png(path, render(fluid, cam, width, height))
            paths.append(path)
            last = t
    return paths
