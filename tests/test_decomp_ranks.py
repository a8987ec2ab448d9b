"""The decomposition's partition and halo bookkeeping, as separate ranks on CPU.

Two processes over gloo each hold one block of a lattice in a padded box, as
the reference's ranks do (src/mpi_view_transfer.cpp).  Every step they
collide their interior with the oracle, exchange the 26 halo messages the
library's plan describes (imex_decomp_halo: peers, boxes, and only the
directions that cross each channel - 9 / 3 / 1), and pull-stream from the
padded box.  The gathered field must equal the undivided oracle run bit for
bit: the plan's boxes, peers and pruned direction sets are exactly what the
pull needs.  The plan's rank grids are the ones the reference itself chose
(tests/golden/reference_runs.json).
"""
import json
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

from conftest import GOLDEN, ROOT

DECK = "1.0  0.1  400\n0.06  12  6\n12  10  16\n"


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _box(F, dirs, lo, ext):
    return F[list(dirs), lo[0]:lo[0] + ext[0], lo[1]:lo[1] + ext[1], lo[2]:lo[2] + ext[2]]


def _rank_main(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import torch
    import torch.distributed as dist

    import imexlbm_gb300 as m
    from oracle import oracle as o
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        d = o.parse_deck(DECK)
        n = (d.sx, d.sy, d.sz)
        E = o.velocities()
        blk = m.decomp_block(world, *n, rank)
        lo, L = blk["lo"], blk["len"]
        F = np.zeros((27, L[0] + 2, L[1] + 2, L[2] + 2))
        F[:, 1:-1, 1:-1, 1:-1] = o.init(*n, d.rho0, d.u0)[:, lo[0]:lo[0] + L[0], lo[1]:lo[1] + L[1],
                                                           lo[2]:lo[2] + L[2]]
        plan = [m.decomp_halo(world, *n, rank, c) for c in range(26)]
        for _ in range(d.Time):
            inner = np.ascontiguousarray(F[:, 1:-1, 1:-1, 1:-1])
            o.collide(inner, d.tau)
            F[:, 1:-1, 1:-1, 1:-1] = inner
            # the halo: send my boundary box on side `offset`, receive my ghost box on side -offset
            reqs, inbox = [], {}
            for c, msg in enumerate(plan):
                out = _box(F, msg["dirs"], msg["send_lo"], msg["ext"]).copy()
                if msg["send_to"] == rank and msg["recv_from"] == rank:
                    inbox[c] = out
                    continue
                recv = torch.empty(out.size, dtype=torch.float64)
                reqs.append(dist.isend(torch.from_numpy(out.ravel()), msg["send_to"], tag=c))
                reqs.append(dist.irecv(recv, msg["recv_from"], tag=c))
                inbox[c] = recv
            for r in reqs:
                r.wait()
            for c, msg in enumerate(plan):
                box = inbox[c]
                box = box if isinstance(box, np.ndarray) else box.numpy()
                lo_r, ext = msg["recv_lo"], msg["ext"]
                F[list(msg["dirs"]), lo_r[0]:lo_r[0] + ext[0], lo_r[1]:lo_r[1] + ext[1],
                  lo_r[2]:lo_r[2] + ext[2]] = box.reshape(len(msg["dirs"]), *ext)
            # pull streaming from the padded box
            G = np.empty((27, *L))
            for a in range(27):
                x0, y0, z0 = 1 - E[a, 0], 1 - E[a, 1], 1 - E[a, 2]
                G[a] = F[a, x0:x0 + L[0], y0:y0 + L[1], z0:z0 + L[2]]
            F[:, 1:-1, 1:-1, 1:-1] = G
        q.put((rank, lo, L, np.ascontiguousarray(F[:, 1:-1, 1:-1, 1:-1])))
    finally:
        dist.destroy_process_group()


def test_two_ranks_exchange_the_pruned_halo_and_match_the_oracle(oracle, imex):
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    parts = [q.get(timeout=300) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    d = oracle.parse_deck(DECK)
    f = oracle.init(d.sx, d.sy, d.sz, d.rho0, d.u0)
    oracle.step(f, d.tau, d.Time)
    got = np.full_like(f, np.nan)
    for _, lo, L, block in parts:
        got[:, lo[0]:lo[0] + L[0], lo[1]:lo[1] + L[1], lo[2]:lo[2] + L[2]] = block
    assert imex.decomp_grid(world, d.sx, d.sy, d.sz) != (1, 1, 1)
    assert np.array_equal(got, f)


def test_plan_grids_are_the_references():
    import imexlbm_gb300 as m
    with open(os.path.join(GOLDEN, "reference_runs.json")) as fp:
        runs = json.load(fp)
    for name, rec in runs["decks"].items():
        n = [int(v) for v in rec["deck"].split()[6:9]]
        for ranks, run in rec["runs"].items():
            g = m.decomp_grid(int(ranks), *n)
            assert run["layout"] == "rx=%d,ry=%d,rz=%d" % g, (name, ranks)


@pytest.mark.parametrize("nranks,n", [(6, (18, 20, 22)), (8, (32, 32, 32)), (5, (7, 9, 30)), (12, (13, 17, 19))])
def test_plan_is_consistent(imex, nranks, n):
    """Blocks tile the lattice; every channel's message is the one its peer
    expects; the pruned sets are 9 / 3 / 1 directions crossing the channel."""
    from oracle import oracle as o
    E = o.velocities()
    cover = np.zeros(n, dtype=int)
    blocks = [imex.decomp_block(nranks, *n, r) for r in range(nranks)]
    for b in blocks:
        lo, L = b["lo"], b["len"]
        cover[lo[0]:lo[0] + L[0], lo[1]:lo[1] + L[1], lo[2]:lo[2] + L[2]] += 1
        g = imex.decomp_grid(nranks, *n)
        c = b["coord"]
        assert b["rank"] == c[0] + g[0] * c[2] + g[0] * g[2] * c[1]
    assert (cover == 1).all()
    for r in range(nranks):
        for ch in range(26):
            msg = imex.decomp_halo(nranks, *n, r, ch)
            peer = imex.decomp_halo(nranks, *n, msg["send_to"], ch)
            assert peer["recv_from"] == r
            assert peer["ext"] == msg["ext"]
            off = np.array(msg["offset"])
            nz = int(np.count_nonzero(off))
            assert len(msg["dirs"]) == {1: 9, 2: 3, 3: 1}[nz]
            for a in msg["dirs"]:
                assert all(E[a, k] == off[k] for k in range(3) if off[k] != 0)
