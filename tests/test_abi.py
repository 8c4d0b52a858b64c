"""The C-ABI library builds, loads and exports every symbol the header
declares (no compute calls: these run without a GPU)."""
import os
import re

from conftest import REPO


def _declared():
    names = []
    for fn in os.listdir(os.path.join(REPO, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(REPO, "include", fn)).read()
            names += re.findall(r"^\s*(?:int|const char\*)\s+(ps_\w+)\s*\(", src, re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = _declared()
    assert "ps_step_rk4" in names and "ps_plan_create" in names and len(names) >= 12


def test_library_exports_declared_symbols(built_lib):
    from phrike_gb300 import _lib
    for name in _declared():
        assert hasattr(built_lib, name), name
    assert set(_declared()) <= set(_lib.exported_names())


def test_error_paths_without_device(built_lib):
    import ctypes as C
    from phrike_gb300 import _lib
    desc = _lib.PlanDesc()
    assert built_lib.ps_plan_desc_init(C.byref(desc), 3) == 0
    desc.n[0] = desc.n[1] = desc.n[2] = 14  # 2 * 7: no pencil transform for the factor 7
    h = C.c_void_p()
    rc = built_lib.ps_plan_create(C.byref(desc), C.byref(h))
    assert rc == 2 and b"N=14" in built_lib.ps_last_error()
    desc.ndim = 4
    assert built_lib.ps_plan_create(C.byref(desc), C.byref(h)) == 1
    size = C.c_size_t()
    assert built_lib.ps_plan_desc_init(C.byref(desc), 3) == 0
    desc.n[0] = desc.n[1] = desc.n[2] = 256
    assert built_lib.ps_plan_scratch_bytes(C.byref(desc), C.byref(size)) == 0
    assert size.value >= 35 * 256 ** 3 * 4


def test_lgl_descriptor_validation_without_device(built_lib):
    """LGL x LGL descriptors are validated before any device work."""
    import ctypes as C
    from phrike_gb300 import _lib
    desc = _lib.PlanDesc()
    h = C.c_void_p()
    size = C.c_size_t()
    assert built_lib.ps_plan_desc_init(C.byref(desc), 2) == 0
    assert desc.gemm_precision == _lib.PS_GEMM_FP32
    desc.n[0], desc.n[1] = 257, 257
    desc.length[0] = desc.length[1] = 2.0
    desc.basis[0] = _lib.PS_BASIS_LEGENDRE
    assert built_lib.ps_plan_create(C.byref(desc), C.byref(h)) == 2  # hybrid basis
    assert b"mixed" in built_lib.ps_last_error()
    desc.basis[1] = _lib.PS_BASIS_LEGENDRE
    assert built_lib.ps_batch_scratch_bytes(C.byref(desc), 3, C.byref(size)) == 0
    assert size.value >= 3 * 16 * 257 * 257 * 4 + 2 * 12 * 257 * 257
    desc.gemm_precision = 7
    assert built_lib.ps_plan_create(C.byref(desc), C.byref(h)) == 1
    desc.gemm_precision = _lib.PS_GEMM_BF16X3
    desc.n[1] = 2
    assert built_lib.ps_plan_create(C.byref(desc), C.byref(h)) == 2
    assert built_lib.ps_plan_desc_init(C.byref(desc), 3) == 0
    for a in range(3):
        desc.n[a] = 17
        desc.basis[a] = _lib.PS_BASIS_LEGENDRE
    assert built_lib.ps_plan_create(C.byref(desc), C.byref(h)) == 2  # 3D Legendre
    assert built_lib.ps_lgl_build(1, 2.0, None, None, None, None) == 1


def test_mixed_radix_descriptor_validation_without_device(built_lib):
    """Fourier axes of any 2^a 3^b 5^c length up to 4096 validate (the
    khi2d_4k grid 3840 x 2160 among them); other factors, lengths above 4096,
    MHD and artificial viscosity on such axes are refused before any device
    work, and so is the static right-hand side."""
    import ctypes as C
    from phrike_gb300 import _lib
    desc = _lib.PlanDesc()
    size = C.c_size_t()
    h = C.c_void_p()
    assert built_lib.ps_plan_desc_init(C.byref(desc), 2) == 0
    desc.n[0], desc.n[1] = 3840, 2160
    assert built_lib.ps_batch_scratch_bytes(C.byref(desc), 1, C.byref(size)) == 0
    assert size.value >= 16 * 3840 * 2160 * 4
    for n in (48, 96, 384, 45, 15, 6, 4096, 3000):
        assert built_lib.ps_plan_desc_init(C.byref(desc), 1) == 0
        desc.n[0] = n
        assert built_lib.ps_plan_scratch_bytes(C.byref(desc), C.byref(size)) == 0, n
    for n in (14, 4100, 5120, 1):
        desc.n[0] = n
        assert built_lib.ps_plan_scratch_bytes(C.byref(desc), C.byref(size)) == 2, n
    assert built_lib.ps_plan_desc_init(C.byref(desc), 2) == 0
    desc.n[0], desc.n[1] = 48, 48
    desc.equations = _lib.PS_EQ_MHD
    assert built_lib.ps_plan_create(C.byref(desc), C.byref(h)) == 2
    assert b"power-of-two" in built_lib.ps_last_error()
    desc.equations = _lib.PS_EQ_EULER
    desc.av_mode = _lib.PS_AV_SENSOR
    assert built_lib.ps_plan_create(C.byref(desc), C.byref(h)) == 2
    assert b"viscosity" in built_lib.ps_last_error()
    desc.av_mode = _lib.PS_AV_OFF
    fake = C.c_void_p(256)  # never dereferenced: the call is refused first
    assert built_lib.ps_rhs_static(C.byref(desc), fake, fake, None) == 2
    assert b"powers of two" in built_lib.ps_last_error()


def test_scratch_accounts_for_the_split_2d_right_hand_side(built_lib):
    """From 256 rows (n[1]) the 2D Euler and MHD last pass is split and keeps
    its right-hand side in a scratch buffer of 4 (Euler) or 8 (MHD) fields;
    HBM admission reads these bytes.  Swapping the axes of a 256 x 128 grid
    changes nothing else in the count."""
    import ctypes as C
    from phrike_gb300 import _lib
    cells = 256 * 128
    for eq, extra in ((_lib.PS_EQ_EULER, 4), (_lib.PS_EQ_MHD, 8)):
        sizes = []
        for nx, ny in ((256, 128), (128, 256)):
            desc = _lib.PlanDesc()
            assert built_lib.ps_plan_desc_init(C.byref(desc), 2) == 0
            desc.equations = eq
            desc.n[0], desc.n[1] = nx, ny
            size = C.c_size_t()
            assert built_lib.ps_batch_scratch_bytes(C.byref(desc), 2, C.byref(size)) == 0
            sizes.append(size.value)
        assert sizes[1] - sizes[0] == extra * cells * 4 * 2, (eq, sizes)


def test_scratch_accounts_for_the_second_3d_stage_input(built_lib):
    """3D Euler with gravity keeps a second 5-field stage input (stages 1 and
    2 must not read and write one buffer); mixed-radix 3D plans need none."""
    import ctypes as C
    from phrike_gb300 import _lib

    def size(n, grav):
        desc = _lib.PlanDesc()
        assert built_lib.ps_plan_desc_init(C.byref(desc), 3) == 0
        desc.n[0] = desc.n[1] = desc.n[2] = n
        desc.gravity[2] = grav
        out = C.c_size_t()
        assert built_lib.ps_batch_scratch_bytes(C.byref(desc), 3, C.byref(out)) == 0
        return out.value

    assert size(32, -1.0) - size(32, 0.0) == 5 * 32 ** 3 * 4 * 3
    assert size(48, -1.0) == size(48, 0.0)
