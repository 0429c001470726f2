"""Argument checks of the extended Python API, without a GPU.

The structured, Fourier, batch and sampling entry points reject malformed
input before any device work, with the reference's error types where the
reference has the same argument (src/lib.rs:33-84: TypeError for a wrong
array type or dimensionality, a ValueError for the shape asserts of
src/field.rs:44-46, 104-106, 223-225) and ValueError for the extensions'
own options.
"""
import numpy as np
import pytest


def _modes(n=10, d=3):
    rng = np.random.default_rng(0)
    return rng.normal(size=(d, n)), rng.standard_normal(n), rng.standard_normal(n)


def test_structured_axes_checks(gsc):
    cov, z1, z2 = _modes()
    with pytest.raises(ValueError):
        gsc.summate_structured(cov, z1, z2, (np.arange(4.0), np.arange(5.0)))      # 2 axes for d=3
    with pytest.raises(TypeError):
        gsc.summate_structured(cov, z1, z2, (np.arange(4.0), np.arange(5.0), [1.0, 2.0]))
    with pytest.raises(TypeError):
        gsc.summate_structured(cov, z1, z2, (np.arange(4), np.arange(5.0), np.arange(6.0)))
    with pytest.raises(ValueError):
        gsc.summate_structured(cov, z1[:9], z2, (np.arange(4.0),) * 3)
    with pytest.raises(ValueError):
        gsc.summate_incompr_structured(*_modes(d=1), (np.arange(4.0),))


def test_fourier_checks(gsc):
    cov, z1, z2 = _modes(d=2)
    pos = np.zeros((2, 7))
    with pytest.raises(ValueError):
        gsc.summate_fourier(np.ones(9), cov, z1, z2, pos)          # spectrum factor length
    with pytest.raises(TypeError):
        gsc.summate_fourier(np.ones((10, 1)), cov, z1, z2, pos)
    with pytest.raises(ValueError):
        gsc.summate_fourier(np.ones(10), cov, z1, z2, np.zeros((3, 7)))


def test_batch_checks(gsc):
    cov, z1, z2 = _modes()
    item = {"cov": cov, "z1": z1, "z2": z2, "pos": np.zeros((3, 4))}
    with pytest.raises(ValueError):
        gsc.summate_batch([dict(item, kind="spectral")])
    with pytest.raises(ValueError):
        gsc.summate_batch([dict(item, pos=np.zeros((2, 4)))])
    with pytest.raises(ValueError):
        gsc.summate_batch([dict(item, z1=z1[:5])])
    with pytest.raises(TypeError):
        gsc.summate_batch([dict(item, z2=z2.astype(np.float32))])
    with pytest.raises(KeyError):
        gsc.summate_batch([dict(item, kind="fourier")])            # no spectrum_factor


def test_sampling_checks(gsc):
    with pytest.raises(ValueError):
        gsc.sample_modes("matern", 2, 10, 1.0, 0)


def test_data_address_of_any_layout():
    """The Python layer's data address agrees with numpy's for C-ordered,
    Fortran-ordered, strided, offset, empty and read-only arrays."""
    import numpy as np
    import gstools_core as gsc
    a = np.arange(12.0).reshape(3, 4)
    ro = a.copy()
    ro.setflags(write=False)
    for x in (a, np.asfortranarray(a), a[:, ::2], a[1:], a[::-1], np.zeros(0), ro):
        assert gsc._ptr(x) == x.ctypes.data
