"""CPU tests of the C ABI library: it builds, loads, and exports every symbol
declared in include/evoc_gb300.h. No compute call is made without a GPU."""
import ctypes
import re
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT, ensure_library


def declared_functions() -> list[str]:
    text = (ROOT / "include" / "evoc_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^EVOC_API\s+(?:const\s+)?\w+\*?\s+\*?(evoc_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declarations_found():
    names = declared_functions()
    assert "evoc_fuzzy_set" in names and "evoc_embed" in names and len(names) >= 15


def test_library_exports_every_declared_symbol():
    lib = ensure_library()
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib)], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_python_binding_lists_every_symbol():
    import evoc_gb300 as E
    assert sorted(E.EXPORTED) == declared_functions()


def test_load_and_abi_version():
    ensure_library()
    import evoc_gb300 as E
    lib = E.load_library()
    assert lib.evoc_abi_version() == 1


def test_default_params_match_reference():
    """EvocEmbeddingParams::default, src/graph/mod.rs:52-67."""
    ensure_library()
    import evoc_gb300 as E
    lib = E.load_library()
    p = E.EmbedParamsC()
    lib.evoc_embed_params_default(ctypes.byref(p))
    assert (p.n_epochs, p.noise_level, p.negative_sample_rate, p.initial_alpha) == (50, 0.5, 1.0,
                                                                                       pytest.approx(0.1))
    assert p.beta1 == 0.5 and p.beta2 == pytest.approx(0.9) and p.eps == pytest.approx(1e-7)
    d = E.EvocEmbeddingParams()
    assert (d.n_epochs, d.noise_level, d.beta1) == (50, 0.5, 0.5)


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="a GPU is present")
def test_context_fails_loudly_without_gpu():
    ensure_library()
    import evoc_gb300 as E
    with pytest.raises(E.EvocError) as ei:
        E.Context(0)
    assert ei.value.code in (E.EVOC_ERR_NO_DEVICE, E.EVOC_ERR_CUDA)


def test_null_context_arguments_rejected():
    ensure_library()
    import evoc_gb300 as E
    lib = E.load_library()
    h = ctypes.c_void_p()
    assert lib.evoc_fuzzy_set(None, None, None, 0, 0, 0.0, 1, ctypes.byref(h)) == E.EVOC_ERR_INVALID_ARGUMENT
    assert lib.evoc_ctx_create(0, None) != 0
    assert lib.evoc_last_error(None) is not None


def test_null_handles_rejected_by_the_newer_entry_points():
    """The warm-start, kNN-handoff, partition, self-test, autotuner,
    initialisation and MST entry points reject NULL handles with
    EVOC_ERR_INVALID_ARGUMENT before any device work."""
    ensure_library()
    import evoc_gb300 as E
    lib = E.load_library()
    h = ctypes.c_void_p()
    bad = E.EVOC_ERR_INVALID_ARGUMENT
    k = ctypes.c_int64()
    loss = (ctypes.c_float * 1)()
    p = E.MlpTrainParams().to_c()
    assert lib.evoc_mlp_create(None, 64, 64, 8, 0, ctypes.byref(h)) == bad
    assert lib.evoc_mlp_get_params(None, None) == bad
    assert lib.evoc_mlp_set_params(None, None) == bad
    assert lib.evoc_mlp_predict(None, None, 0, None) == bad
    assert lib.evoc_mlp_predict_device(None, None, 0, None) == bad
    assert lib.evoc_mlp_gradients(None, None, None, 1, loss, None) == bad
    assert lib.evoc_mlp_fit_device(None, 1, None, None, None, ctypes.byref(p), None) == bad
    assert lib.evoc_mlp_n_params(None) == 0
    lib.evoc_mlp_free(None)  # no-op
    assert lib.evoc_to_bf16_device(None, None, 0, None) == bad
    assert lib.evoc_fuzzy_set_device_raw(None, None, None, 0, 2, 1, 1.0, 1, ctypes.byref(h)) == bad
    assert lib.evoc_label_prop_partition(None, None, 1, 1, 0, None, ctypes.byref(k)) == bad
    assert lib.evoc_selftest_wait_timeout(None, 10) == bad
    assert "NULL" in lib.evoc_last_error(None).decode() or lib.evoc_last_error(None)
    # the autotuner, the bisection-work counter, the label-propagation
    # initialisation and the minimum spanning tree
    assert lib.evoc_plan_set_config(None, 0, 2, 0) == bad
    assert lib.evoc_plan_autotune(None, None, None) == bad
    assert lib.evoc_ctx_smooth_knn_steps(None, ctypes.byref(k)) == bad
    assert lib.evoc_label_propagation_init(None, None, 8, None, 0, 0, None) == bad
    assert lib.evoc_label_propagation_init_device(None, None, 8, None, 0, 0, None) == bad
    assert lib.evoc_build_mst(None, None, 10, 4, 5, None, None, None, ctypes.byref(k)) == bad
    assert lib.evoc_build_mst_device(None, None, 10, 4, 5, None, None, None,
                                     ctypes.byref(k)) == bad


def test_mlp_train_params_default():
    """evoc_mlp_train_params_default fills the documented defaults (no GPU)."""
    import ctypes as C
    import evoc_gb300 as E
    p = E.MlpTrainParamsC()
    E.load_library().evoc_mlp_train_params_default(C.byref(p))
    d = E.MlpTrainParams()
    assert (p.steps, p.batch, p.align_every, p.align_rows) == (d.steps, d.batch, d.align_every,
                                                               d.align_rows)
    for name in ("lr", "beta1", "beta2", "eps", "lr_end"):
        assert getattr(p, name) == pytest.approx(getattr(d, name), rel=1e-6), name
    assert p.seed == d.seed
