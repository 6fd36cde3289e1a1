"""Host replica of the tensor-core operand packing (schur_tc.cu): a
K-major, no-swizzle tcgen05 descriptor reads core matrices of 8 rows x 16
bytes, the two core matrices of a K-step `lbo` bytes apart and successive
8-row groups `sbo` bytes apart.  Reading the packed A' / B'' tiles that way
must give the real matrices whose product is the complex Schur update."""
import numpy as np

TILE_M, TILE_NC, PANEL = 128, 32, 64


def pack_off(r, k, groups):
    s, ki, e, mi, rr = k >> 3, (k >> 2) & 1, k & 3, r >> 3, r & 7
    return s * (2 * groups * 128) + ki * (groups * 128) + mi * 128 + rr * 16 + e * 4


def descriptor_read(buf, rows, groups, step, lbo, sbo):
    """The (rows x 128) K-major matrix an MMA sequence sees, K-step by K-step."""
    out = np.zeros((rows, 2 * PANEL), np.float32)
    for s in range(2 * PANEL // 8):
        base = s * step
        for m in range(rows):
            for k in range(8):
                off = base + (k // 4) * lbo + (m // 8) * sbo + (m % 8) * 16 + (k % 4) * 4
                out[m, 8 * s + k] = buf[off // 4]
    return out


def test_packed_tiles_form_the_complex_product():
    rng = np.random.default_rng(0)
    L = (rng.standard_normal((TILE_M, PANEL)) + 1j * rng.standard_normal((TILE_M, PANEL))).astype(np.complex64)
    U = (rng.standard_normal((PANEL, TILE_NC)) + 1j * rng.standard_normal((PANEL, TILE_NC))).astype(np.complex64)
    ga, gb = TILE_M // 8, 2 * TILE_NC // 8
    A = np.zeros(TILE_M * 2 * PANEL, np.float32)
    B = np.zeros(2 * TILE_NC * 2 * PANEL, np.float32)
    for r in range(TILE_M):
        for l in range(PANEL):
            A[pack_off(r, 2 * l, ga) // 4] = L[r, l].real
            A[pack_off(r, 2 * l + 1, ga) // 4] = L[r, l].imag
    for j in range(TILE_NC):
        for l in range(PANEL):
            re, im = U[l, j].real, U[l, j].imag
            B[pack_off(2 * j, 2 * l, gb) // 4] = re
            B[pack_off(2 * j, 2 * l + 1, gb) // 4] = -im
            B[pack_off(2 * j + 1, 2 * l, gb) // 4] = im
            B[pack_off(2 * j + 1, 2 * l + 1, gb) // 4] = re
    Am = descriptor_read(A, TILE_M, ga, 2 * ga * 128, ga * 128, 128)        # M x K'
    Bm = descriptor_read(B, 2 * TILE_NC, gb, 2 * gb * 128, gb * 128, 128)  # N' x K' (K-major B)
    D = Am.astype(np.float64) @ Bm.astype(np.float64).T                     # M x N'
    C = L.astype(np.complex128) @ U.astype(np.complex128)
    assert np.allclose(D[:, 0::2], C.real, rtol=1e-5, atol=1e-4)
    assert np.allclose(D[:, 1::2], C.imag, rtol=1e-5, atol=1e-4)
    assert max(pack_off(TILE_M - 1, 2 * PANEL - 1, ga), pack_off(2 * TILE_NC - 1, 2 * PANEL - 1, gb)) < 65536
