"""Sharding reconstructions across processes (one GPU each).

Two partitions of the work, as the reference's MPI tools split it:

- by view block (tools/pjrec.cpp:375-418): the reference's MPI pjrec scatters
  contiguous view blocks (MPIWorld's work-unit split: nView/P views each, the
  first nView%P ranks one more, tools/mpiworld.cpp:42-63), backprojects them
  locally and sums the partial images (ReduceImageMPI).  Here each rank
  filters and backprojects its block without PostProcessing, the partial
  images are summed with one all-reduce, and the rotation scale is applied
  once.  (The reference's MPI build scales each partial image by
  pi/nView_local, over-scaling the sum by P; the single-process result is the
  one reproduced here.)  `reconstruct_sharded` does one slice,
  `reconstruct_views_batch` a batch of slices of one geometry.
- by problem (tools/phm2pj.cpp:404-433 splits ray-sums by view in the same
  way; independent slices need no exchange at all): `problem_block` gives each
  rank a contiguous range of the batch's slices.

The image sum uses the process group's backend: NCCL sums device tensors in
place; with gloo (CPU ranks, or several processes sharing one GPU in tests)
the partial image is summed in host memory and copied back.
"""


def view_block(n_view, rank, world):
    """[start, count) of `rank`'s contiguous view block."""
    per, extra = divmod(n_view, world)
    start = rank * per + min(rank, extra)
    return start, per + (1 if rank < extra else 0)


def problem_block(n_problems, rank, world):
    """[start, count) of `rank`'s contiguous range of problems (slices)."""
    return view_block(n_problems, rank, world)


def reduce_partial_images(image, group=None):
    """Sum partial (un-post-processed) images over the process group in place.
    `image` is a torch tensor (device or host)."""
    import torch.distributed as dist
    if not dist.is_initialized() or dist.get_world_size(group) <= 1:
        return image
    if image.is_cuda and dist.get_backend(group) != "nccl":
        host = image.cpu()
        dist.all_reduce(host, op=dist.ReduceOp.SUM, group=group)
        image.copy_(host)
    else:
        dist.all_reduce(image, op=dist.ReduceOp.SUM, group=group)
    return image


def reconstruct_sharded(plan, sino, angles, image, rank, world, group=None):
    """Each rank filters and backprojects its view block of one slice, the
    images are summed, then PostProcessing scales once.
    plan: ctsim_gb300.device.ReconPlan; sino [n_view, pitch] / image [nx, ny]:
    CUDA tensors."""
    start, count = view_block(len(angles), rank, world)
    if count > 0:
        plan.run(sino, angles, image, start_view=start, n_views=count, postprocess=False)
    else:
        image.zero_()
    reduce_partial_images(image, group)
    plan.postprocess(image)
    return image


def reconstruct_views_batch(plan, block, angles, start, filtered, images, group=None,
                            stream=None):
    """One rank's share of a batch of slices sharded by view block.

    block [B, count, pitch]: this rank's views [start, start + count) of every
    slice, contiguous (what the rank was sent); filtered: scratch of the same
    shape; images [B, nx, ny].  One filter launch over the B x count rows, one
    batched backprojection of them without PostProcessing, the image sum over
    the group, then PostProcessing of every slice."""
    import numpy as np
    B, count, pitch = block.shape
    ang = np.ascontiguousarray(angles[start:start + count], np.float64)
    if count > 0:
        plan.filter(block.view(B * count, pitch), filtered.view(B * count, pitch), stream=stream)
        plan.backproject_batch(filtered, ang, images, postprocess=False, stream=stream)
    else:
        images.zero_()
    reduce_partial_images(images, group)
    for b in range(B):
        plan.postprocess(images[b], stream=stream)
    return images
