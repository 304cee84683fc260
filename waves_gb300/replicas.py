"""Independent replicas on N GPUs.

The solver step has no data-parallel exchange on one GPU's domain (it would need a halo exchange
per kernel if the domain were decomposed), so N GPUs run N independent simulations, one per rank
of the default process group, and the whole job's figures are aggregated here: simulated seconds
add up, device and end-to-end wall seconds are bounded by the slowest rank.
"""


def aggregate(sim_s, device_s, e2e_sim_s=0.0, e2e_wall_s=0.0, device=None):
    """(total simulated s, max device s, total e2e simulated s, max e2e wall s) over the ranks."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(sim_s), float(device_s), float(e2e_sim_s), float(e2e_wall_s)
    total = torch.tensor([sim_s, e2e_sim_s], dtype=torch.float64, device=device)
    worst = torch.tensor([device_s, e2e_wall_s], dtype=torch.float64, device=device)
    dist.all_reduce(total, op=dist.ReduceOp.SUM)
    dist.all_reduce(worst, op=dist.ReduceOp.MAX)
    return total[0].item(), worst[0].item(), total[1].item(), worst[1].item()
