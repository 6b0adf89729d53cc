"""CPU oracle of the reference's particle inflow (test infrastructure only).

CMultiGPUHandler::InsertBucket, radix/SPVSOLVER/MultiGPUSolver/MultiGPUHandler.cpp:
1163-1210, restated on the set of IDs in use: the handler's output slots
0 .. ParticleNum-1 are indexed by ID and a slot whose ID is negative is a hole (a
particle removed by CCellSet::CheckParticleOutsideComputeZone).  Bucket particles fill
the holes in increasing slot order and take the slot as their ID; when the bucket
outlasts the holes, the rest is appended at ParticleNum.. only if
ParticleNum + (rest) <= MaxParticleNum (:1189), otherwise it is not added.
"""


def insert_bucket(ids_in_use, extent, max_particles, count):
    """Returns (IDs given to bucket particles 0, 1, ... in order, new extent)."""
    used = set(int(i) for i in ids_in_use)
    out = []
    for i in range(extent):
        if len(out) == count:
            break
        if i not in used:
            out.append(i)
    rest = count - len(out)
    if rest > 0 and extent + rest <= max_particles:
        out.extend(range(extent, extent + rest))
        extent += rest
    return out, extent
