"""Multi-GPU layout of the FX path: replicas only.

The F-engine is independent per (element, spectrum), the X-engine per
channel, and integrations are independent once each carries its Ntaps-1
spectra of PFB history.  Splitting channels across GPUs would need an
all-to-all corner turn (ReorderFOutput across devices,
MDT_device_functions.cu:183-208), so the work is split by integration (one
stream) or by job (ragged batches) instead: every rank runs the single-GPU
path on its own share, with no collective on the data path.  The only
collective is an optional host-side gather of results at the end.

This module holds that host logic: the split, the input span each rank needs
(its own integrations plus the lead-in spectra), a cost-balanced job split,
and the gather.  It uses torch.distributed only for the gather.
"""


def integration_split(nint_total, rank, world):
    """Contiguous share of `nint_total` integrations: (first, count); the
    first nint_total % world ranks take one more."""
    if world < 1 or not 0 <= rank < world or nint_total < 0:
        raise ValueError("bad split")
    base, extra = divmod(nint_total, world)
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def input_span(first, count, nspectra, ntaps):
    """Spectra of I/Q a rank needs for integrations [first, first + count):
    (first spectrum, number of spectra).  Integration j of a stream reads
    spectra [j*Nsp, j*Nsp + Nsp + Ntaps - 1) (the lead-in is the previous
    integration's last Ntaps - 1 spectra, MDT_OneStation_client.cu:1170)."""
    if count <= 0:
        return first * nspectra, 0
    return first * nspectra, count * nspectra + ntaps - 1


def job_split(costs, world):
    """Jobs -> ranks by longest-processing-time-first (deterministic: ties
    by job index, then the least-loaded rank with the lowest index).
    Returns a list of job-index lists, one per rank."""
    order = sorted(range(len(costs)), key=lambda j: (-costs[j], j))
    load = [0.0] * world
    out = [[] for _ in range(world)]
    for j in order:
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(j)
        load[r] += costs[j]
    return [sorted(x) for x in out]


def gather_integrations(vis, nint_total, rank, world, root=0, group=None):
    """Gathers each rank's [count, ...] result tensor (from integration_split)
    into one [nint_total, ...] tensor on `root` (None elsewhere).  Complex
    tensors travel as their real view.  Uses padded equal-size gathers."""
    import torch
    import torch.distributed as dist
    cplx = vis.is_complex()
    x = torch.view_as_real(vis) if cplx else vis
    per = -(-nint_total // world)
    pad = torch.zeros((per,) + tuple(x.shape[1:]), dtype=x.dtype, device=x.device)
    pad[:x.shape[0]] = x
    bufs = [torch.empty_like(pad) for _ in range(world)] if rank == root else None
    dist.gather(pad, bufs, dst=root, group=group)
    if rank != root:
        return None
    parts = []
    for r in range(world):
        _, cnt = integration_split(nint_total, r, world)
        parts.append(bufs[r][:cnt])
    out = torch.cat(parts)
    return torch.view_as_complex(out.contiguous()) if cplx else out
