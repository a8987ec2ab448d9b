"""The ticket order of the two-steps-per-launch kernel (k_two_fxs,
imexlbm_gb300/csrc/kernels_fx.cu), restated on the host.

CTAs take tickets in order; a ticket is one row of phase A (step j into the
ring of x-planes) or of phase B (step j + 1 from the ring).  A CTA waits only
for rows of smaller tickets - rows other CTAs took earlier and are running -
so every wait ends: B(x, y) waits for A of rows (x +- 1, y +- 1), and A(x, y)
of a recycled ring slot waits for B of the rows of planes x - R - 1 ..
x - R + 1 that read that slot.  A trails by lag = (R + 1) ny / 2 + 2
tickets (imex two_step_lag).  This checks the order for ring depths 4..16
and a range of lattice shapes, and that every row of both phases has
exactly one ticket.
"""
import pytest

RING = 6  # the default ring depth


def lag_of(ny, ring):
    return (ring + 1) * ny // 2 + 2  # two_step_lag


def decode(t, nx, ny, ring=RING):
    n = nx * ny
    lag, total = lag_of(ny, ring), 2 * n
    if t < lag:
        is_a, r = True, t
    elif t < total - lag:
        u = t - lag
        is_a = bool(u & 1)
        r = lag + (u >> 1) if is_a else u >> 1
    else:
        is_a, r = False, t - n
    if is_a:
        return True, r // ny, r % ny
    p, q = divmod(r, ny)  # planes 1 .. nx-1 then 0; rows 1 .. ny-1 then 0
    return False, (p + 1 if p < nx - 1 else 0), (q + 1 if q < ny - 1 else 0)


def deps(is_a, x, y, nx, ny, ring=RING):
    if not is_a:
        return [(True, (x + dx) % nx, (y + dy) % ny) for dx in (-1, 0, 1) for dy in (-1, 0, 1)]
    if x < ring + 2:
        return []
    return [(False, (x + dx) % nx, (y + dy) % ny) for dx in (-ring - 1, -ring, -ring + 1) for dy in (-1, 0, 1)]


SHAPES = [(8, 4), (9, 5), (13, 7), (16, 16), (32, 32), (40, 23), (64, 9), (128, 128)]


@pytest.mark.parametrize("ring", [4, 6, 12, 16])
@pytest.mark.parametrize("nx,ny", SHAPES)
def test_every_wait_is_on_an_earlier_ticket(nx, ny, ring):
    if lag_of(ny, ring) > nx * ny:
        pytest.skip("refused: the lag exceeds the lattice's rows")
    ticket = {}
    for t in range(2 * nx * ny):
        key = decode(t, nx, ny, ring)
        assert key not in ticket
        ticket[key] = t
    assert len(ticket) == 2 * nx * ny
    slack = min(t - ticket[d] for key, t in ticket.items() for d in deps(*key, nx, ny, ring))
    assert slack >= 1
    if nx >= ring + 4:  # both kinds of wait occur: the lag balances them at about (R - 3) ny / 2
        assert slack >= (ring - 3) * ny // 2 - 1, slack


def test_ring_slot_readers_are_the_awaited_rows():
    """Row y of the slot A(x, y) overwrites held plane x - R, read by B of
    planes x - R - 1 .. x - R + 1, rows y - 1 .. y + 1: exactly the rows it
    waits for."""
    nx, ny = 20, 6
    for x in range(RING + 2, nx):
        for y in range(ny):
            p = x - RING
            readers = {(False, (p + dx) % nx, (y + dy) % ny) for dx in (-1, 0, 1) for dy in (-1, 0, 1)}
            assert set(deps(True, x, y, nx, ny)) == readers
