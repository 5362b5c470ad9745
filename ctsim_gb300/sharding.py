"""View-block sharding of one reconstruction across processes (one GPU each).

The reference's MPI pjrec scatters contiguous view blocks (MPIWorld's
work-unit split: nView/P views each, the first nView%P ranks one more,
tools/mpiworld.cpp:42-63), backprojects them locally and sums the partial
images (tools/pjrec.cpp:375-418).  Here each rank reconstructs its block
without PostProcessing, the partial images are summed with one all-reduce,
and the global rotation scale is applied once.  (The reference's MPI build
scales each partial image by pi/nView_local, over-scaling the sum by P; the
single-process result is the one reproduced here.)
"""


def view_block(n_view, rank, world):
    """[start, count) of `rank`'s contiguous view block."""
    per, extra = divmod(n_view, world)
    start = rank * per + min(rank, extra)
    return start, per + (1 if rank < extra else 0)


def reduce_partial_images(image, group=None):
    """Sum partial (un-post-processed) images over the process group in place.
    `image` is a torch tensor on the device the group's backend uses."""
    import torch.distributed as dist
    if dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(image, op=dist.ReduceOp.SUM, group=group)
    return image


def reconstruct_sharded(plan, sino, angles, image, rank, world, group=None):
    """Each rank backprojects its view block, images are summed, then scaled.
    plan: ctsim_gb300.device.ReconPlan; sino/image: CUDA tensors."""
    start, count = view_block(len(angles), rank, world)
    if count > 0:
        plan.run(sino, angles, image, start_view=start, n_views=count, postprocess=False)
    else:
        image.zero_()
    reduce_partial_images(image, group)
    plan.postprocess(image)
    return image
