"""encode -> erase -> decode round trips on the GPU.

Recovery slices are computed on the GPU; k input slices are then "lost", the
k x k system over GF(2^16) formed by the PAR2 coefficients of k recovery rows
is inverted on the CPU (the oracle's multiply), and the lost slices are
rebuilt with the same GPU multiply-accumulate:

    y_r = rec_r + sum_{i known} c(r,i) in_i          (accumulate onto rec rows)
    in_E = M^-1 y,   M[r][e] = c(r, e)                (explicit coefficients)

Exact reconstruction of every lost byte checks the whole contraction at
sizes where a full CPU recomputation would be slow.
"""
import numpy as np
import pytest

from oracle import oracle as O
from parpar_gb300 import _lib

pytestmark = pytest.mark.gpu


def gf_inv_matrix(M):
    """Inverse of a square matrix over GF(2^16) (Gauss-Jordan, oracle arithmetic)."""
    L = O.lib()
    n = len(M)
    A = [list(map(int, row)) + [1 if i == j else 0 for j in range(n)] for i, row in enumerate(M)]
    for col in range(n):
        piv = next(r for r in range(col, n) if A[r][col])
        A[col], A[piv] = A[piv], A[col]
        inv = next(x for x in range(1, 65536) if L.or_mul(A[col][col], x) == 1) if A[col][col] != 1 else 1
        A[col] = [L.or_mul(v, inv) for v in A[col]]
        for r in range(n):
            if r != col and A[r][col]:
                f = A[r][col]
                A[r] = [a ^ L.or_mul(f, b) for a, b in zip(A[r], A[col])]
    return [row[n:] for row in A]


def gf_inverse_fast(M):
    """Same as gf_inv_matrix with log/exp tables (faster for k ~ 100)."""
    L = O.lib()
    exp = np.array([L.or_exp(v) for v in range(65535)], dtype=np.int64)
    log = np.zeros(65536, dtype=np.int64)
    log[exp] = np.arange(65535)

    def mul_row(row, f):
        out = np.zeros_like(row)
        nz = row != 0
        if f:
            out[nz] = exp[(log[row[nz]] + log[f]) % 65535]
        return out
    n = len(M)
    A = np.concatenate([np.array(M, dtype=np.int64), np.eye(n, dtype=np.int64)], axis=1)
    for col in range(n):
        piv = col + int(np.nonzero(A[col:, col])[0][0])
        A[[col, piv]] = A[[piv, col]]
        inv = exp[(65535 - log[A[col, col]]) % 65535]
        A[col] = mul_row(A[col], int(inv))
        for r in range(n):
            if r != col and A[r, col]:
                A[r] ^= mul_row(A[col], int(A[r, col]))
    return A[:, n:].astype(np.uint16)


def test_small_inverse_agrees():
    rng = np.random.default_rng(1)
    M = rng.integers(1, 65536, size=(4, 4))
    a = np.array(gf_inv_matrix(M), dtype=np.uint16)
    b = gf_inverse_fast(M)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("N,R,S,k,method", [
    (40, 12, 4100, 12, 1),
    (2000, 200, 65536, 200, 1),     # the bandwidth workload's counts, 64 KiB slices, every recovery slice used
    (300, 64, 32768, 50, 4),        # the tensor-core variant
    (4096, 96, 16384, 96, 1),       # the dense workload's input count
])
def test_encode_erase_decode(N, R, S, k, method):
    torch = pytest.importorskip("torch")
    from parpar_gb300.job import par2_coefficients
    L = _lib.load()
    rng = np.random.default_rng(N + R)
    pitch = L.par2cuda_row_pitch_bytes(S)
    pw = pitch // 2
    nw = ((S + 7) // 8 * 8 + 8) // 2
    d_in = torch.empty((N, pw), dtype=torch.int16, device="cuda")
    _lib.check(L.par2cuda_synth_fill(d_in.data_ptr(), pitch, N, S, 99, 0, None), "synth")
    exps = sorted(rng.choice(65535, size=R, replace=False).tolist())
    coeff = par2_coefficients(np.arange(N), exps)                    # [R][N]
    d_coeff = torch.from_numpy(coeff.view(np.int16)).cuda()
    d_rec = torch.empty((R, pw), dtype=torch.int16, device="cuda")
    sb = L.par2cuda_muladd_scratch_bytes(max(R, k), N)
    scratch = torch.empty(sb, dtype=torch.uint8, device="cuda")
    _lib.check(L.par2cuda_muladd(d_in.data_ptr(), pw, N, d_coeff.data_ptr(), d_rec.data_ptr(), pw, R, nw, 0, method,
                                 scratch.data_ptr(), sb, None), "encode")
    # erase k inputs, use k recovery rows
    lost = np.sort(rng.choice(N, size=k, replace=False))
    known = np.setdiff1d(np.arange(N), lost)
    rows = np.sort(rng.choice(R, size=k, replace=False))
    # y = rec[rows] + sum_known c(rows, known) in_known
    d_y = d_rec[torch.from_numpy(rows).cuda()].contiguous()
    d_known = d_in[torch.from_numpy(known).cuda()].contiguous()
    ck = np.ascontiguousarray(coeff[np.ix_(rows, known)])
    d_ck = torch.from_numpy(ck.view(np.int16)).cuda()
    _lib.check(L.par2cuda_muladd(d_known.data_ptr(), pw, len(known), d_ck.data_ptr(), d_y.data_ptr(), pw, k, nw, 1,
                                 method, scratch.data_ptr(), sb, None), "subtract known")
    # x = M^-1 y
    Minv = gf_inverse_fast(coeff[np.ix_(rows, lost)])
    d_minv = torch.from_numpy(np.ascontiguousarray(Minv).view(np.int16)).cuda()
    d_x = torch.empty((k, pw), dtype=torch.int16, device="cuda")
    _lib.check(L.par2cuda_muladd(d_y.data_ptr(), pw, k, d_minv.data_ptr(), d_x.data_ptr(), pw, k, nw, 0, method,
                                 scratch.data_ptr(), sb, None), "solve")
    torch.cuda.synchronize()
    assert L.par2cuda_device_error() == 0
    got = d_x.view(torch.uint8)[:, :S]
    want = d_in.view(torch.uint8)[torch.from_numpy(lost).cuda(), :S]
    assert torch.equal(got, want)
