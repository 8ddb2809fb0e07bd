"""Helpers for GPU parity tests: move batches of column-major matrices between
numpy (layout (batch, ncols, ld), C order) and device memory, build pointer
arrays, plant guard bands, and measure errors against the oracle."""
import numpy as np

EPS = {np.float64: 2.0 ** -53, np.float32: 2.0 ** -24}


def eps(dtype):
    return EPS[np.dtype(dtype).type]


def to_dev(torch, a: np.ndarray):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def ptr_array(torch, t, count: int | None = None):
    """Device array of per-matrix device pointers for a (batch, ncols, ld) tensor."""
    batch = t.shape[0]
    stride = t.stride(0) * t.element_size()
    base = t.data_ptr()
    ptrs = np.array([base + b * stride for b in range(batch if count is None else count)],
                    dtype=np.int64)
    return torch.from_numpy(ptrs).cuda()


def scattered_copies(torch, a: np.ndarray, seed=0):
    """Copy every matrix of a batch into its own device allocation (shuffled
    order inside one pool, with gaps) and return (pool, ptr tensor, offsets)."""
    batch, ncol, ld = a.shape
    per = ncol * ld + 7  # deliberately unaligned gaps
    order = np.random.default_rng(seed).permutation(batch)
    pool = np.full(batch * per + 16, np.nan, dtype=a.dtype)
    offs = np.zeros(batch, dtype=np.int64)
    for slot, b in enumerate(order):
        o = slot * per + 3
        offs[b] = o
        pool[o:o + ncol * ld] = a[b].reshape(-1)
    dpool = torch.from_numpy(pool).cuda()
    ptrs = torch.from_numpy(dpool.data_ptr() + offs * a.itemsize).cuda()
    return dpool, ptrs, offs


def gather_scattered(dpool, offs, shape):
    pool = dpool.cpu().numpy()
    batch, ncol, ld = shape
    out = np.empty(shape, dtype=pool.dtype)
    for b in range(batch):
        out[b] = pool[offs[b]:offs[b] + ncol * ld].reshape(ncol, ld)
    return out


def lower(a: np.ndarray, n: int):
    """Lower triangles (including diagonal) of a (batch, n, ld) column-major
    batch, as (batch, n, n) row-major arrays."""
    m = np.ascontiguousarray(a[:, :n, :n].transpose(0, 2, 1))
    return np.tril(m)


def dense(a: np.ndarray, rows: int, cols: int):
    """(batch, rows, cols) row-major view of a column-major batch."""
    return np.ascontiguousarray(a[:, :cols, :rows].transpose(0, 2, 1))


def sym_from_lower(a: np.ndarray, n: int):
    low = lower(a, n)
    return low + np.tril(low, -1).transpose(0, 2, 1)
