"""MRC2014 result files (utils/data_io.py:50-160 writes them with mrcfile):
header layout, round trips, and MatchTemplateResult export / load."""

import struct

import numpy as np
import pytest
import torch

from leopard_em_gb300 import managers as m
from leopard_em_gb300 import mrc


@pytest.mark.parametrize("shape,dtype", [((7, 9), np.float32), ((3, 5, 6), np.float32), ((4, 4), np.int16),
                                         ((2, 3), np.float16)])
def test_round_trip_and_header(tmp_path, shape, dtype):
    rng = np.random.default_rng(0)
    data = (rng.standard_normal(shape) * 10).astype(dtype)
    path = tmp_path / "a.mrc"
    mrc.write_mrc(path, data, voxel_size=1.5)
    back = mrc.read_mrc(path)
    assert back.dtype == data.dtype and back.shape == data.shape
    np.testing.assert_array_equal(back, data)
    head = path.read_bytes()[:1024]
    nx, ny, nz = struct.unpack_from("<3i", head, 0)
    assert (nz, ny, nx) == ((1,) + shape if len(shape) == 2 else shape)
    assert head[208:212] == b"MAP " and head[212:214] == b"\x44\x44"
    assert struct.unpack_from("<i", head, 108)[0] == 20141
    assert struct.unpack_from("<3i", head, 64) == (1, 2, 3)
    dmin, dmax, dmean = struct.unpack_from("<3f", head, 76)
    assert dmin == pytest.approx(float(data.min()), rel=1e-3) and dmax == pytest.approx(float(data.max()), rel=1e-3)
    assert struct.unpack_from("<3f", head, 40)[0] == pytest.approx(1.5 * nx)
    assert len(path.read_bytes()) == 1024 + data.nbytes


def test_overwrite_and_errors(tmp_path):
    path = tmp_path / "b.mrc"
    mrc.write_mrc(path, torch.zeros(4, 4))
    with pytest.raises(FileExistsError):
        mrc.write_mrc(path, torch.zeros(4, 4))
    mrc.write_mrc(path, torch.ones(4, 4), overwrite=True)
    assert mrc.read_mrc(path).sum() == 16
    with pytest.raises(ValueError):
        mrc.write_mrc(tmp_path / "c.mrc", np.zeros(5))
    (tmp_path / "d.mrc").write_bytes(b"\0" * 100)
    with pytest.raises(ValueError):
        mrc.read_mrc(tmp_path / "d.mrc")


def test_result_export_and_load(tmp_path):
    g = torch.Generator().manual_seed(1)
    maps = {k: torch.rand(12, 10, generator=g) for k in m.MatchTemplateResult.MAPS}
    paths = {f"{k}_path": str(tmp_path / f"{k}.mrc") for k in m.MatchTemplateResult.MAPS}
    r = m.MatchTemplateResult(**maps, **paths)
    r.export_results()
    with pytest.raises(ValueError, match="already exists"):  # the reference refuses existing outputs
        m.MatchTemplateResult(**paths)
    r2 = m.MatchTemplateResult(**paths, allow_file_overwrite=True)
    r2.load_tensors_from_paths()
    for k in m.MatchTemplateResult.MAPS:
        assert torch.equal(getattr(r2, k), maps[k])
    with pytest.raises(FileExistsError):
        r.export_results()
    r.allow_file_overwrite = True
    r.export_results()
    with pytest.raises(ValueError):
        m.MatchTemplateResult(**maps).export_results()
