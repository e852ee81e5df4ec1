"""z-slab decomposition of the TGV-DCT deshade over several ranks (one GPU each).

The reference runs one volume on one device (tgv_cuda/tgv_common.cu:249-253, the
loop at tgv_deshade/tgv2_l1_deshade.cu:169-272).  Here a volume of depth D is split
along z into contiguous slabs, one per rank.  Each rank keeps a context for its own
planes plus one halo plane on each side that has a neighbour, and:

  loop       after every iteration, sends the first own plane's ubar and vbar to the
             rank below (its top halo) and the last own plane's to the rank above (its
             bottom halo).  One iteration of an own plane reads ubar and vbar one plane
             either side, p one plane below and q one plane above.  p at the bottom
             halo and q at the top halo need no exchange: their updates read only
             that plane and the one on the own side (p takes forward differences of
             ubar, q backward differences of vbar), so the halo plane computes them
             exactly.  The halo planes' ubar and vbar are wrong after each local
             iteration (they read the missing plane beyond) and are overwritten by the
             exchange, so every own plane advances exactly as in the single volume;
  Poisson    sends its last own plane's v_z up (the divergence reads v_z one plane
             below), runs the divergence and the forward x, y contractions on its
             planes, transposes its own planes into z pencils (one all-to-all: every
             rank gets all D planes of a span of whole rows), runs the forward z
             contraction, the eigenvalue division and the inverse z contraction on its
             pencil (cosine_transform.cu:198-223 is the reference's z pass), transposes
             back (the second all-to-all) and runs the inverse y, x contractions.

The single-volume solve runs its passes in the same order (forward x, y, z, inverse z,
y, x), and every value is the same dot product summed in the same order, so u, v and l
equal the single-volume results bit for bit (FP32 state, FP32 contractions).

One algorithm (`deshade_rank`, a generator that yields its communication requests)
serves two drivers: `run_distributed` over torch.distributed (NCCL between GPUs, or
gloo), and `run_emulated`, which runs every rank's generator in one process and hands
the messages over directly.  The compute is a backend object: `CudaSlabBackend` calls
the C ABI (tgvdct_state_*_dev, tgvdct_tgv2_step_dev, tgvdct_slab_poisson_*_dev,
tgvdct_pencil_*); anything with the same methods can stand in for it.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

# field-mask bits of the loop state (include/tgvdct.h)
FIELD_F = 1 << 0
FIELD_U = 1 << 1
FIELD_V = 7 << 2
FIELD_V_Z = 1 << 4
FIELD_UBAR = 1 << 5
FIELD_VBAR = 7 << 6
FIELD_P = 7 << 9
FIELD_Q = 63 << 12
# what a rank's halo planes receive from its neighbours after every iteration
HALO_FIELDS = FIELD_UBAR | FIELD_VBAR


def field_count(mask: int) -> int:
    return bin(mask).count("1")


def split_evenly(n: int, parts: int):
    """[(begin, end)] of `parts` contiguous ranges covering 0..n, sizes differing by
    at most one, the larger ones first."""
    if parts < 1 or n < parts:
        raise ValueError(f"cannot split {n} into {parts} non-empty ranges")
    q, r = divmod(n, parts)
    out, b = [], 0
    for k in range(parts):
        e = b + q + (1 if k < r else 0)
        out.append((b, e))
        b = e
    return out


@dataclass(frozen=True)
class SlabGeometry:
    """Rank `rank` of `ranks` for a width x height x depth volume."""
    width: int
    height: int
    depth: int
    ranks: int
    rank: int

    @property
    def z_range(self):
        return split_evenly(self.depth, self.ranks)[self.rank]

    @property
    def below(self) -> int:  # halo planes under the own planes (0 or 1)
        return 1 if self.rank > 0 else 0

    @property
    def above(self) -> int:
        return 1 if self.rank < self.ranks - 1 else 0

    @property
    def own_planes(self) -> int:
        z0, z1 = self.z_range
        return z1 - z0

    @property
    def local_depth(self) -> int:
        return self.own_planes + self.below + self.above

    @property
    def local_z_range(self):
        """Global planes held locally (own planes and halos)."""
        z0, z1 = self.z_range
        return z0 - self.below, z1 + self.above

    def column_range(self, rank=None):
        """Columns (of the W*H plane, whole rows) of a rank's z pencil."""
        rows = split_evenly(self.height, self.ranks)[self.rank if rank is None else rank]
        return rows[0] * self.width, rows[1] * self.width

    def check(self):
        if self.ranks < 1 or not 0 <= self.rank < self.ranks:
            raise ValueError("rank out of range")
        if self.depth < 2 * self.ranks or self.height < self.ranks:
            raise ValueError("a z-slab split needs depth >= 2 * ranks and height >= ranks")


def deshade_rank(geo: SlabGeometry, backend, f_local, iterations: int, *,
                 set_negative_values_to_zero: bool = False):
    """One rank's deshade as a generator of communication requests.

    Yields ("halo", send_down, send_up, n_below, n_above): the planes for the rank
    below and above (None where nothing goes there) and the number of values expected
    from the rank below and above (None where nothing comes); expects (from_below,
    from_above) back.  Yields ("alltoall", chunks) with one chunk per destination rank
    and expects the list of chunks received, by source rank.  Returns (u, v_x, v_y,
    v_z, l, r) of the rank's own planes."""
    import torch

    geo.check()
    W, H, D = geo.width, geo.height, geo.depth
    Dl, lo = geo.local_depth, geo.below
    first, last = lo, lo + geo.own_planes - 1
    n_halo = field_count(HALO_FIELDS) * W * H
    backend.init(f_local)
    for _ in range(iterations):
        backend.step()
        send_down = backend.read(HALO_FIELDS, first) if geo.below else None
        send_up = backend.read(HALO_FIELDS, last) if geo.above else None
        from_below, from_above = yield ("halo", send_down, send_up,
                                        n_halo if geo.below else None,
                                        n_halo if geo.above else None)
        if from_below is not None:
            backend.write(HALO_FIELDS, 0, from_below)
        if from_above is not None:
            backend.write(HALO_FIELDS, Dl - 1, from_above)
    # the divergence reads v_z one plane below
    send_up = backend.read(FIELD_V_Z, last) if geo.above else None
    from_below, _ = yield ("halo", None, send_up, W * H if geo.below else None, None)
    if from_below is not None:
        backend.write(FIELD_V_Z, 0, from_below)
    u, vx, vy, vz = backend.read_all(FIELD_U | FIELD_V).view(4, Dl, H, W).unbind(0)
    rhs = backend.poisson_xy(vx, vy, vz)  # (Dl, H, W): divergence, forward x, forward y
    own = slice(lo, lo + geo.own_planes)
    mine = rhs[own].reshape(geo.own_planes, H * W)
    # slab -> pencils: rank s gets this rank's planes of its columns
    chunks = []
    for s in range(geo.ranks):
        c0, c1 = geo.column_range(s)
        chunks.append(mine[:, c0:c1].contiguous())
    got = yield ("alltoall", chunks)
    pencil = torch.cat([g.reshape(-1) for g in got]).reshape(D, -1)  # sources in z order
    c0, c1 = geo.column_range()
    pencil = backend.pencil_z(pencil, c0)  # forward z, division, inverse z
    # pencils -> slab: rank s gets its planes of this rank's columns
    chunks = []
    for s in range(geo.ranks):
        z0, z1 = split_evenly(D, geo.ranks)[s]
        chunks.append(pencil[z0:z1].contiguous())
    got = yield ("alltoall", chunks)
    back = torch.empty(geo.own_planes, H * W, dtype=mine.dtype, device=mine.device)
    for s, g in enumerate(got):
        a, b = geo.column_range(s)
        back[:, a:b] = g.reshape(geo.own_planes, b - a)
    l = backend.poisson_inverse_yx(back.reshape(geo.own_planes, H, W), D)
    u_own = u[own]
    r = u_own - l
    if set_negative_values_to_zero:
        r = torch.clamp_min(r, 0.0)
    return u_own, vx[own], vy[own], vz[own], l, r


def run_emulated(gens):
    """Drives every rank's generator in one process, in lock step, handing each
    message straight to its receiver.  Returns the ranks' results."""
    n = len(gens)
    reqs = [g.send(None) for g in gens]
    results = [None] * n
    while True:
        live = [k for k in range(n) if results[k] is None]
        if not live:
            return results
        kinds = {reqs[k][0] for k in live}
        if len(kinds) != 1 or len(live) != n:
            raise RuntimeError("ranks out of step")
        kind = kinds.pop()
        replies = []
        for k in range(n):
            if kind == "halo":
                from_below = reqs[k - 1][2] if k > 0 else None
                from_above = reqs[k + 1][1] if k < n - 1 else None
                replies.append((from_below, from_above))
            else:
                replies.append([reqs[s][1][k] for s in range(n)])
        for k in range(n):
            try:
                reqs[k] = gens[k].send(replies[k])
            except StopIteration as stop:
                results[k] = stop.value


def run_distributed(gen, rank: int, ranks: int, group=None):
    """Drives this rank's generator with torch.distributed: point-to-point sends and
    receives for the halos, all_to_all_single for the pencil transpositions."""
    req = gen.send(None)
    while True:
        if req[0] == "halo":
            reply = _halo_exchange(req, rank, ranks, group)
        else:
            reply = _all_to_all(req[1], group)
        try:
            req = gen.send(reply)
        except StopIteration as stop:
            return stop.value


def _halo_exchange(req, rank, ranks, group):
    """Sends a rank's halo planes to its neighbours and receives theirs (sizes known
    to both sides), as one batch of point-to-point operations."""
    import torch
    import torch.distributed as dist

    _, send_down, send_up, n_below, n_above = req
    ref = send_down if send_down is not None else send_up
    if ref is not None:
        device = ref.device
    elif dist.get_backend(group) == "nccl":  # a rank that only receives
        device = torch.device("cuda", torch.cuda.current_device())
    else:
        device = torch.device("cpu")
    ops, from_below, from_above = [], None, None
    if send_down is not None:
        ops.append(dist.P2POp(dist.isend, send_down.contiguous(), rank - 1, group))
    if send_up is not None:
        ops.append(dist.P2POp(dist.isend, send_up.contiguous(), rank + 1, group))
    if n_below is not None:
        from_below = torch.empty(n_below, dtype=torch.float32, device=device)
        ops.append(dist.P2POp(dist.irecv, from_below, rank - 1, group))
    if n_above is not None:
        from_above = torch.empty(n_above, dtype=torch.float32, device=device)
        ops.append(dist.P2POp(dist.irecv, from_above, rank + 1, group))
    for w in dist.batch_isend_irecv(ops) if ops else []:
        w.wait()
    return from_below, from_above


def _all_to_all(chunks, group):
    """One all_to_all_single: chunks[s] goes to rank s; returns the chunks received,
    by source rank.  Chunk sizes are exchanged first."""
    import torch
    import torch.distributed as dist

    device = chunks[0].device
    n = len(chunks)
    send_sizes = torch.tensor([c.numel() for c in chunks], dtype=torch.int64, device=device)
    recv_sizes = torch.empty(n, dtype=torch.int64, device=device)
    dist.all_to_all_single(recv_sizes, send_sizes, group=group)
    rs = [int(x) for x in recv_sizes.tolist()]
    flat = torch.cat([c.reshape(-1) for c in chunks])
    out = torch.empty(sum(rs), dtype=flat.dtype, device=device)
    dist.all_to_all_single(out, flat, output_split_sizes=rs,
                           input_split_sizes=[c.numel() for c in chunks], group=group)
    return list(torch.split(out, rs))


# ---------------------------------------------------------------------------
class CudaSlabBackend:
    """A rank's slab on the GPU: a context of the local shape (own planes and halos)
    and, for its z pencil, a tgvdct_pencil of the whole volume's depth.  FP32 state
    and FP32 contractions (the combination whose results the slab split reproduces
    bit for bit)."""

    def __init__(self, params, geo: SlabGeometry):
        import copy

        import torch

        from . import Context, DCT_FP32, STATE_FP32, lib
        if params.state_precision != STATE_FP32 or params.dct_mode != DCT_FP32:
            raise ValueError("the slab split runs FP32 state and FP32 contractions")
        self.geo = geo
        self.params = copy.copy(params)
        self.params.depth = geo.local_depth
        self.device = torch.device("cuda", torch.cuda.current_device())
        self.ctx = Context(self.params)
        self._lib = lib
        self._pencil = None
        self.W, self.H = geo.width, geo.height
        self.Dl = geo.local_depth

    @property
    def stream(self):
        """torch's current stream on this device: the library's calls and the torch
        operations of the driver (slicing, concatenation) stay in one order."""
        import torch
        return torch.cuda.current_stream(self.device).cuda_stream

    def close(self):
        if self._pencil:
            self._lib().tgvdct_pencil_destroy(self._pencil)
            self._pencil = None
        self.ctx.close()

    def _check(self, st):
        from . import _check
        _check(st, allow_stop=False)

    def init(self, f_local):
        self._check(self._lib().tgvdct_state_init_dev(self.ctx._ctx, f_local.data_ptr(),
                                                      self.stream))

    def step(self):
        self._check(self._lib().tgvdct_tgv2_step_dev(self.ctx._ctx, 1, self.stream))

    def _read(self, mask, plane, count):
        import torch
        out = torch.empty(field_count(mask) * count * self.W * self.H, dtype=torch.float32,
                          device=self.device)
        self._check(self._lib().tgvdct_state_read_dev(self.ctx._ctx, mask, plane, count,
                                                      out.data_ptr(), self.stream))
        return out

    def read(self, mask, plane):
        return self._read(mask, plane, 1)

    def read_all(self, mask):
        return self._read(mask, 0, self.Dl)

    def write(self, mask, plane, buf):
        buf = buf.contiguous()
        self._check(self._lib().tgvdct_state_write_dev(self.ctx._ctx, mask, plane, 1,
                                                       buf.data_ptr(), self.stream))

    def poisson_xy(self, vx, vy, vz):
        import torch
        out = torch.empty(self.Dl, self.H, self.W, dtype=torch.float32, device=self.device)
        vx, vy, vz = (t.contiguous() for t in (vx, vy, vz))
        self._check(self._lib().tgvdct_slab_poisson_xy_dev(
            self.ctx._ctx, vx.data_ptr(), vy.data_ptr(), vz.data_ptr(), out.data_ptr(),
            self.stream))
        return out

    def pencil_z(self, pencil, column_begin):
        import torch
        D, cols = pencil.shape
        if self._pencil is None:
            p = ctypes.c_void_p()
            self._check(self._lib().tgvdct_pencil_create(self.W, self.H, D, cols,
                                                         ctypes.byref(p)))
            self._pencil = p
        pencil = pencil.contiguous()
        out = torch.empty_like(pencil)
        self._check(self._lib().tgvdct_pencil_poisson_z_dev(
            self._pencil, pencil.data_ptr(), out.data_ptr(), column_begin,
            self.params.poisson_eigen, self.stream))
        return out

    def poisson_inverse_yx(self, own, total_depth):
        import torch
        own = own.contiguous()
        out = torch.empty_like(own)
        self._check(self._lib().tgvdct_slab_poisson_inverse_yx_dev(
            self.ctx._ctx, own.data_ptr(), out.data_ptr(), own.shape[0], total_depth,
            self.stream))
        return out


def local_input(f, geo: SlabGeometry):
    """The planes of a whole volume f (D, H, W) that rank geo.rank holds."""
    z0, z1 = geo.local_z_range
    part = f[z0:z1]
    return part.contiguous() if hasattr(part, "contiguous") else part.copy()
