"""Generates srgb_tables.inc: the exact sRGB8 quantisation tables of the engine.

The reference converts shaded colours with unPremultLinearToSRGB followed by
packUnorm4x8 (shaders/shaderCommon.glsl:61-71, shaders/oitSimple.frag.glsl:53-55)
and back with unPremultSRGBToLinear (shaderCommon.glsl:83-93). This engine
quantises with the exact threshold of each 8-bit code instead of a float pow,
so that the CPU oracle and the CUDA kernels pick the same code for every input:

  thr[k]    (k = 0..254) smallest float c with enc(c)*255 >= k + 0.5,
            enc evaluated in double; thr[255] = 3e38 sentinel.
  bucket[i] (i = 0..4095) code of c = i/4096, so that
            code(c) = bucket[floor(c*4096)] + (c >= thr[bucket[...]]).
  dec[k]    linear value of sRGB code k, rounded to float.

Run: python gen_srgb_tables.py > srgb_tables.inc
"""
import math
import struct
import sys


def enc(c):
    if c < 0.0031308:
        return c * 12.92
    return math.pow(c, 1.0 / 2.4) * 1.055 - 0.055


def b2f(b):
    return struct.unpack('<f', struct.pack('<I', b))[0]


def f2b(f):
    return struct.unpack('<I', struct.pack('<f', f))[0]


def thresholds():
    out = []
    for k in range(255):
        target = (k + 0.5) / 255.0
        lo, hi = 0, 0x3F800000
        while lo < hi:
            mid = lo + (hi - lo) // 2
            if enc(b2f(mid)) >= target:
                hi = mid
            else:
                lo = mid + 1
        out.append(b2f(lo))
    return out


def code_of(c, thr):
    lo, hi = 0, 255
    while lo < hi:
        mid = (lo + hi) >> 1
        if c >= thr[mid]:
            lo = mid + 1
        else:
            hi = mid
    return lo


def decode(k):
    s = k / 255.0
    return s / 12.92 if s < 0.04045 else math.pow((s + 0.055) / 1.055, 2.4)


def main(out=sys.stdout):
    thr = thresholds()
    bucket = [code_of(b2f(f2b(i / 4096.0)), thr) for i in range(4096)]
    dec = [b2f(f2b(decode(k))) for k in range(256)]
    w = out.write
    w('// Generated by gen_srgb_tables.py; do not edit.\n')
    w('#define OIT_SRGB_THR_INIT { \\\n')
    for k in range(255):
        w('  %s, \\\n' % (float.hex(thr[k]) + 'f'))
    w('  3.0e38f }\n')
    w('#define OIT_SRGB_BUCKET_INIT { \\\n')
    for i in range(0, 4096, 32):
        w('  ' + ', '.join(str(v) for v in bucket[i:i + 32]) + ', \\\n')
    w('}\n')
    w('#define OIT_SRGB_DEC_INIT { \\\n')
    for k in range(256):
        w('  %s, \\\n' % (float.hex(dec[k]) + 'f'))
    w('}\n')


if __name__ == '__main__':
    main()
