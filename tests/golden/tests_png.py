"""Minimal PNG reader (8-bit RGB/RGBA, non-interlaced) for comparing against image files."""
import struct, zlib, numpy as np
def read_png(path):
    b = open(path,'rb').read()
    assert b[:8] == b'\x89PNG\r\n\x1a\n'
    pos = 8; idat = b''; w=h=None
    while pos < len(b):
        ln, = struct.unpack('>I', b[pos:pos+4]); t = b[pos+4:pos+8]; d = b[pos+8:pos+8+ln]; pos += 12+ln
        if t == b'IHDR': w,h,bd,ct,_,_,il = struct.unpack('>IIBBBBB', d); assert bd==8 and il==0; ch = {2:3,6:4}[ct]
        elif t == b'IDAT': idat += d
    raw = zlib.decompress(idat); stride = w*ch
    out = np.zeros((h, stride), np.uint8); prev = np.zeros(stride, np.int32)
    for y in range(h):
        f = raw[y*(stride+1)]; line = np.frombuffer(raw[y*(stride+1)+1:(y+1)*(stride+1)], np.uint8).astype(np.int32)
        cur = np.zeros(stride, np.int32)
        if f == 0: cur = line
        elif f == 2: cur = (line + prev) & 255
        else:
            for x in range(stride):
                a = cur[x-ch] if x >= ch else 0; c = prev[x-ch] if x >= ch else 0; up = prev[x]
                if f == 1: v = line[x] + a
                elif f == 3: v = line[x] + ((a + up) >> 1)
                elif f == 4:
                    p = a + up - c; pa, pb, pc = abs(p-a), abs(p-up), abs(p-c)
                    pr = a if (pa <= pb and pa <= pc) else (up if pb <= pc else c); v = line[x] + pr
                cur[x] = v & 255
        out[y] = cur; prev = cur
    return out.reshape(h, w, ch)
