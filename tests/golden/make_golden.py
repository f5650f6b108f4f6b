"""Writes the golden fixtures of the reference's test sequence.

For each of the 93 cases of the reference's test.py (13-51), rendered by the
CPU oracle at 64x40 with the reference's scene and state: the RGBA8 image
and the fragment count. tests/test_golden.py checks the oracle against them
bit for bit (CPU) and the engine within 1 LSB (GPU).

  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, 'oracle'))

import oracle as orc  # noqa: E402
from vk_order_independent_transparency_gb300 import sequence as sq  # noqa: E402

W, H = 64, 40
PATH = os.path.join(HERE, 'sequence_64x40.npz')


def render(st):
    v, i, tpo = sq.scene(st)
    kw = sq.state_kwargs(st)
    kw.pop('interlock_is_ordered')
    fr = orc.render(st.algorithm, W, H, sq.camera(W, H), v, i, tpo, st.percentTransparent, **kw)
    img, _ = fr.composite()
    return img, fr.fragment_count()


def main():
    names, imgs, frags = [], [], []
    for name, st in sq.cases():
        img, n = render(st)
        names.append(name)
        imgs.append(img)
        frags.append(n)
    np.savez_compressed(PATH, names=np.array(names), images=np.stack(imgs), fragments=np.array(frags, np.uint64),
                        width=W, height=H)
    print(PATH, os.path.getsize(PATH))


if __name__ == '__main__':
    main()
