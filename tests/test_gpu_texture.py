"""fnGenPreviewTextureDevice against the oracle: the Node Editor's preview image
(NoiseTexture::BuildTexture) is the tree wrapped in a default ConvertRGBA8 over a grid centred on
the view offset; pixels and OutputMinMax must equal the oracle's bit for bit."""
import numpy as np
import pytest

from oracle.oracle import OracleTree
from oracle.tree import N
from tests import trees
from tests.parity import minmax_equal

pytestmark = pytest.mark.gpu
F = np.float32


def oracle_texture(root, gen_type, size, offset, scale, seed):
    wrap = N("ConvertRGBA8", Source=root)
    sx, sy = size
    x0 = F(F(offset[0]) - F(F(F(sx) / F(2.0)) * F(scale)))
    y0 = F(F(offset[1]) - F(F(F(sy) / F(2.0)) * F(scale)))
    o = OracleTree(wrap)
    if gen_type == 0:
        return o.grid((x0, y0), (sx, sy), (scale, scale), seed)
    if gen_type == 1:
        return o.tileable(sx, sy, scale, scale, seed)
    if gen_type == 2:
        return o.grid((x0, y0, offset[2]), (sx, sy, 1), (scale,) * 3, seed)
    return o.grid((x0, y0, offset[2], offset[3]), (sx, sy, 1, 1), (scale,) * 4, seed)


@pytest.mark.parametrize("gen_type", [0, 1, 2, 3])
@pytest.mark.parametrize("size, offset, scale", [((64, 48), (10.25, -3.5, 7.0, 2.0), 0.5), ((33, 17), (0, 0, 0, 0), 3.0)])
def test_preview_texture_matches_oracle(gpu, gen_type, size, offset, scale):
    torch = pytest.importorskip("torch")
    fn = gpu
    root = N("FractalFBm", Source=N("Simplex", Feature_Scale=20.0), Octaves=3)
    node = trees.to_product(root)
    n = size[0] * size[1]
    pix = torch.zeros(n, dtype=torch.int32, device="cuda")
    mm = torch.zeros(2, dtype=torch.float32, device="cuda")
    fn.gen_preview_texture(node, gen_type, size, offset, scale, 1337, pix.data_ptr(), mm.data_ptr())
    torch.cuda.synchronize()
    got = pix.cpu().numpy().view(np.uint32)
    o, omm = oracle_texture(root, gen_type, size, offset, scale, 1337)
    assert np.array_equal(got, np.asarray(o, np.float32).view(np.uint32))
    assert (got >> 24 == 255).all()                                   # alpha
    assert ((got & 0xFF) == ((got >> 8) & 0xFF)).all()                # grey
    assert minmax_equal(tuple(mm.cpu().numpy()), omm)
