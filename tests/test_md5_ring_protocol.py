"""A model of the shared-memory ring of the staged file MD5 kernel
(parpar_gb300/csrc/k_hash.cu: k_file_md5_staged), run on the CPU: one chain's
bulk copies of P2C_STG_CH-byte chunks (never crossing a row of sliceBytes,
rounded up to 16 bytes) into P2C_STG_NS slots, each completing on its own
mbarrier in any order; the chain waits on a slot's barrier with the slot's
phase bit, hashes the chunk's full 64-byte blocks, keeps a partial last block
for the finish, and refills the slot while bytes are left.  Every byte of the
file must reach the hash once and in order, every wait must be on a slot with
a copy in flight (so a bounded wait never runs out in a correct run), no copy
may land in a slot before the chain has read its previous chunk, and every
copy must stay inside the file's rows."""
import random

CH = 1024
NS = 3


def run_chain(total, slice_bytes, pitch, rng):
    file_bytes = bytes(rng.getrandbits(8) for _ in range(total))
    rows = [file_bytes[r * slice_bytes:(r + 1) * slice_bytes] for r in range(-(-total // slice_bytes) or 1)]
    state = {"row": 0, "off": 0, "left": total}
    slots = [None] * NS           # chunk bytes once landed
    sizes = [0] * NS
    inflight = {}                 # slot -> bytes still to land
    read = [True] * NS            # the chain has read the slot's last chunk
    phase = [0] * NS              # completed phases per slot
    waited = [0] * NS

    def issue(s):
        assert read[s], "copy into a slot whose chunk was not read yet"
        row_bytes = min(state["left"] + state["off"], slice_bytes)
        size = min(CH, row_bytes - state["off"])
        csize = (size + 15) & ~15
        assert state["off"] + csize <= pitch, "copy past the row's pitch"
        src = rows[state["row"]][state["off"]:state["off"] + size]
        inflight[s] = src
        read[s] = False
        state["left"] -= size
        state["off"] += size
        if state["off"] == row_bytes:
            state["row"] += 1
            state["off"] = 0
        return size

    def land_some():
        # copies complete in any order
        if inflight and rng.random() < 0.7:
            s = rng.choice(sorted(inflight))
            slots[s] = inflight.pop(s)
            phase[s] += 1

    for k in range(NS):
        if state["left"]:
            sizes[k] = issue(k)
    hashed = bytearray()
    tail = b""
    pending = sum(1 for k in range(NS) if k in inflight)
    slot = 0
    steps = 0
    while pending > 0:
        # bounded wait on this slot's next phase
        assert slot in inflight or phase[slot] > waited[slot], "wait on a slot with nothing in flight"
        while phase[slot] == waited[slot]:
            land_some()
            steps += 1
            assert steps < 10 ** 6
        waited[slot] += 1
        pending -= 1
        chunk = slots[slot]
        size = sizes[slot]
        assert len(chunk) == size
        full = size // 64
        hashed += chunk[:full * 64]
        if size % 64:
            assert state["left"] == 0, "a partial block before the file's end"
            tail = chunk[full * 64:]
        read[slot] = True
        if state["left"]:
            sizes[slot] = issue(slot)
            pending += 1
        slot = (slot + 1) % NS
        land_some()
    assert not inflight
    assert bytes(hashed) + tail == file_bytes


def test_md5_ring_protocol():
    rng = random.Random(5)
    for slice_bytes in (64, 128, 960, 1024, 1088, 2048, 4160, 65536):
        pitch = (slice_bytes + 8 + 127) // 128 * 128   # par2cuda_row_pitch_bytes: data, checksum block, 128-byte rows
        for _ in range(12):
            total = rng.choice([1, 15, 63, 64, 65, slice_bytes - 1, slice_bytes, slice_bytes + 1,
                                rng.randint(1, 5 * slice_bytes)])
            total = max(1, total)
            run_chain(total, slice_bytes, pitch, rng)
