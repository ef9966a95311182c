"""Slab decomposition and the z-slab <-> y-slab all-to-all transposes
(incompact3d_gb300/decomp.py), the sharded form of the reference's 2DECOMP
transposes, run as gloo ranks on CPU:

* index maps: balanced blocks, remainder to the first ranks, empty blocks;
* z_to_y / y_to_z reproduce the global field's blocks exactly (ragged sizes,
  a rank without planes, trailing dimensions);
* a compact z-derivative done the sharded way (z-slab -> y-slab, the line
  operator on full z lines, back) equals the single-rank result bit for bit
  (the oracle supplies the line operator: the module only moves data);
* a 3-D FFT done the sharded way (x, y passes on z-slabs, one transpose, z
  pass) equals numpy's fftn to round-off, the Poisson solver's pattern;
* the diagnostics sum over ranks."""
import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
from incompact3d_gb300.decomp import Slabs, block_range  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_block_ranges_cover_the_axis():
    for n in (0, 1, 2, 5, 7, 64, 129):
        for size in (1, 2, 3, 4, 8):
            rs = [block_range(n, size, r) for r in range(size)]
            assert rs[0][0] == 0 and rs[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(rs, rs[1:]))
            lens = [e - s for s, e in rs]
            assert max(lens) - min(lens) <= 1 and lens == sorted(lens, reverse=True)
    with pytest.raises(ValueError):
        block_range(4, 2, 2)


def test_single_rank_transposes_are_identities():
    s = Slabs(5, 4, 3, 0, 1)
    a = torch.arange(60, dtype=torch.float64).reshape(3, 4, 5)
    assert torch.equal(s.z_to_y(a), a) and torch.equal(s.y_to_z(a), a)
    with pytest.raises(ValueError):
        s.z_to_y(a[:2])


def _field(nx, ny, nz, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((nz, ny, nx))


def _cases(rank, ws):
    import torch.distributed as dist
    from incompact3d_gb300.decomp import allreduce_sum
    out = {}
    # exact block moves, ragged sizes and a rank with no planes (nz < ws)
    ok = True
    for (nx, ny, nz) in ((8, 7, 5), (6, 3, 2), (4, 5, 9), (3, 1, 4)):
        g = torch.from_numpy(_field(nx, ny, nz, nx * ny * nz))
        s = Slabs(nx, ny, nz, rank, ws)
        z0, z1 = s.z_slab
        y0, y1 = s.y_slab
        a = g[z0:z1].contiguous()
        b = s.z_to_y(a)
        ok &= torch.equal(b, g[:, y0:y1])
        ok &= torch.equal(s.y_to_z(b), a)
        # a trailing dimension (a complex field as real pairs)
        gc = torch.stack([g, -g], dim=-1)
        bc = s.z_to_y(gc[z0:z1].contiguous())
        ok &= torch.equal(bc, gc[:, y0:y1])
        ok &= torch.equal(s.y_to_z(bc), gc[z0:z1])
    out["blocks"] = bool(ok)
    # sharded 3-D FFT: x, y passes on z-slabs, transpose, z pass
    nx, ny, nz = 16, 12, 10
    g = _field(nx, ny, nz, 7)
    s = Slabs(nx, ny, nz, rank, ws)
    z0, z1 = s.z_slab
    y0, y1 = s.y_slab
    f2 = np.fft.fft2(g[z0:z1], axes=(1, 2))
    b = s.z_to_y(torch.view_as_real(torch.from_numpy(np.ascontiguousarray(f2))).contiguous())
    f3 = np.fft.fft(torch.view_as_complex(b.contiguous()).numpy(), axis=0)
    ref = np.fft.fftn(g)[:, y0:y1]
    out["fft"] = float(np.abs(f3 - ref).max() / np.abs(ref).max()) if ref.size else 0.0
    # diagnostics: kinetic-energy-like sum over ranks
    t = torch.tensor([float((g[z0:z1] ** 2).sum())], dtype=torch.float64)
    allreduce_sum(t)
    out["sum"] = float(abs(t.item() - (g ** 2).sum()) / (g ** 2).sum())
    dist.barrier()
    return out


def _derz_case(rank, ws):
    import oracle
    from conftest import fourier_field
    n = (16, 10, 32)
    L = 2 * np.pi
    o = oracle.Oracle(*n, L, L, L)
    g = fourier_field(*n, seed=3)
    s = Slabs(*n, rank, ws)
    z0, z1 = s.z_slab
    y0, y1 = s.y_slab
    b = s.z_to_y(torch.from_numpy(g[z0:z1].copy())).numpy()
    db = o.op(2, oracle.OP_DER1, 1, b)  # full z lines of this rank's y rows
    dz = s.y_to_z(torch.from_numpy(db)).numpy()
    ref = o.op(2, oracle.OP_DER1, 1, g)[z0:z1]
    return {"derz_equal": bool(np.array_equal(dz, ref))}


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        res = _cases(rank, ws)
        res.update(_derz_case(rank, ws))
        q.put((rank, res))
    except Exception as e:  # reported to the parent, which fails the test
        q.put((rank, {"error": repr(e)}))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("ws", [2, 3])
def test_sharded_transposes_derivative_and_fft_on_gloo_ranks(oracle_mod, ws):
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in range(ws):
        r = res[rank]
        assert "error" not in r, r
        assert r["blocks"], (rank, r)
        assert r["fft"] < 1e-13, (rank, r)
        assert r["sum"] < 1e-13, (rank, r)
        assert r["derz_equal"], (rank, r)
