"""The ranged sweeps' task partition, checked on the host by
cesa_self_test_partition with the same functions the kernels use
(csrc/cesa_sweep.cuh): equal shares and the SM pairs' unequal split (the
EM-ICP forward splits at 208/256, the adjoint's ranged layout at 193/256).
Needs no GPU."""
import ctypes

import numpy as np


def check(cesa, nblk, nch, grid, pair_num):
    k = ctypes.c_int(0)
    rc = cesa.lib().cesa_self_test_partition(nblk, nch, grid, pair_num, ctypes.byref(k))
    return rc, k.value


def test_partition_at_config_3(cesa):
    # forward: 314 owned blocks of 128 rows x 79 chunks of 512 points over 304 blocks
    assert check(cesa, 314, 79, 304, 0) == (cesa.CESA_OK, 2)
    assert check(cesa, 314, 79, 304, 208) == (cesa.CESA_OK, 3)
    # adjoint: 27 column blocks of 1536 x 157 chunks of 256 rows
    assert check(cesa, 27, 157, 304, 193) == (cesa.CESA_OK, 13)


def test_partition_random_shapes(cesa):
    rng = np.random.default_rng(5)
    for _ in range(300):
        grid = 2 * int(rng.integers(1, 161))
        nblk = int(rng.integers(1, 200))
        nch = int(rng.integers(1, 160))
        pn = int(rng.choice([0, 1, 128, 192, 193, 208, 224, 255]))
        rc, kmax = check(cesa, nblk, nch, grid, pn)
        assert rc == cesa.CESA_OK, (nblk, nch, grid, pn)
        assert kmax >= 1


def test_partition_rejects_bad_arguments(cesa):
    assert check(cesa, 10, 10, 7, 208)[0] == cesa.CESA_ERR_INVALID_ARGUMENT  # pairs need an even grid
    assert check(cesa, 10, 10, 8, 256)[0] == cesa.CESA_ERR_INVALID_ARGUMENT
    assert check(cesa, 0, 10, 8, 0)[0] == cesa.CESA_ERR_INVALID_ARGUMENT
