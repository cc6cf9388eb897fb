"""Host-side Python pieces that need no GPU: the warm-start network's
parameter layout and stored model, the command-line seed generator and the
bench's clock record."""
import numpy as np


def test_warmstart_parameter_layout(tmp_path):
    from geogram_gb300 import _lib, warmstart as ws
    p = ws.init_params(seed=3)
    assert p.shape == (_lib.MLP_PARAMS,) and p.dtype == np.float32
    u = ws.unpack(p)
    assert u["W1"].shape == (ws.H, ws.IN) and u["W2"].shape == (ws.H, ws.H)
    assert u["W4"].shape == (ws.H,) and u["b4"].shape == (1,)
    # the padded input columns start (and must stay) at zero
    assert np.all(p[ws.OFF_W1:ws.OFF_B1].reshape(ws.H, 32)[:, ws.IN:] == 0.0)
    m = ws.WarmStartModel(p)
    path = tmp_path / "m.npz"
    m.save(str(path), note="x")
    m2 = ws.WarmStartModel.load(str(path))
    assert np.array_equal(m2.params, m.params) and np.array_equal(m2.norm, m.norm)


def test_shipped_model_loads():
    import json
    from geogram_gb300 import _lib, warmstart as ws
    m = ws.WarmStartModel.load()
    assert m.params.shape == (_lib.MLP_PARAMS,) and m.norm.shape == (_lib.MLP_NORM,)
    assert np.all(np.isfinite(m.params)) and np.all(m.norm[ws.IN:2 * ws.IN] > 0)
    rep = json.loads(str(np.load(ws.DEFAULT_MODEL)["report"]))
    assert rep["loss_last"] < rep["loss_first"]


def test_cli_seed_generator():
    from geogram_gb300.cli import seeds
    u = seeds(1000, 0, 0.05, 1)
    assert u.shape == (1000, 3) and np.all((u >= 0) & (u < 1))
    g = seeds(5000, 8, 0.05, 1)
    assert g.shape == (5000, 3) and np.all((g > 0) & (g < 1))
    h = seeds(5000, 32, 0.05, 1, (0.01, 0.1))
    assert h.shape == (5000, 3) and np.all((h > 0) & (h < 1))
    assert np.array_equal(seeds(100, 4, 0.05, 7), seeds(100, 4, 0.05, 7))


def test_bench_clock_summary_reports_throttle_reasons():
    """The bench's clock record: median SM clock under load, and every
    throttle reason seen active in any sample."""
    import bench
    cs = bench.ClockSampler(0)
    assert cs.summary()["reasons"] == ["no nvidia-smi samples"]
    off = ["Not Active"] * 4
    cs.samples = [["0", "2070", "2070", "900.5", "0x0", *off],
                  ["0", "1980", "2070", "1400.0", "0x4", *off[:3], "Active"],
                  ["0", "2070", "2070", "1000.0", "0x8", "Active", *off[:3]]]
    s = cs.summary()
    assert s["sm_mhz"] == 2070 and s["sm_max_mhz"] == 2070 and s["samples"] == 3
    assert s["reasons"] == ["hw_slowdown", "sw_power_cap"]


def test_device_argument_check():
    """Device entry points get raw pointers: the wrappers refuse host tensors,
    other dtypes, wrong shapes and non-contiguous views before any call."""
    import pytest
    import torch
    import geogram_gb300 as g
    assert g._dev_arg(None, "w", 5) is None
    x = torch.zeros((5, 3), dtype=torch.float64)
    for bad, kw in ((x, dict(cols=3)),                                  # host memory
                    (x.float(), dict(cols=3)),
                    (x.t(), dict(cols=3)),
                    (x[:, 0], dict(n=5))):
        with pytest.raises(ValueError):
            g._dev_arg(bad, "t", **kw)


def test_device_argument_must_be_on_the_context_device():
    """A CUDA tensor on another GPU than the context's is refused before
    its pointer reaches a kernel (stand-ins: no GPU is needed)."""
    import types

    import pytest
    import geogram_gb300 as g

    class FakeCuda:
        is_cuda = True
        dtype = "torch.float64"
        shape = (5, 3)

        def __init__(self, index):
            self.device = types.SimpleNamespace(index=index)

        def is_contiguous(self):
            return True

    ctx0 = types.SimpleNamespace(device=0)
    assert g._dev_arg(FakeCuda(0), "x", cols=3, ctx=ctx0) is not None
    with pytest.raises(ValueError, match="cuda:1"):
        g._dev_arg(FakeCuda(1), "x", cols=3, ctx=ctx0)
