"""PAR2 packets of a create job assembled from GPU results: the index file
(Main, FileDesc, IFSC, Creator) and the recovery packets, whose MD5s are
computed on the GPU; checked by an independent parse and against the oracle."""
import hashlib
import struct

import numpy as np
import pytest

from oracle import oracle as O
from parpar_gb300 import par2packets as P
from parpar_gb300 import synth

pytestmark = pytest.mark.gpu


def test_par2_set_from_gpu_results():
    torch = pytest.importorskip("torch")
    from parpar_gb300.job import ResidentJob, file_layout
    S = 8192
    file_lens = [S * 5 + 1234, 100, 40000, S * 2]
    names = ["data.bin", "small.txt", "médias.iso", "b"]
    first, lens = file_layout(file_lens, S)
    N = len(lens)
    host = np.zeros((N, S), np.uint8)
    files = []
    for f, ln in enumerate(file_lens):
        data = synth.slice_bytes(300 + f, 0, ln)
        files.append(data)
        for k in range((ln + S - 1) // S):
            chunk = data[k * S:(k + 1) * S]
            host[first[f] + k, :len(chunk)] = chunk
    exps = [0, 1, 2, 7, 100]
    job = ResidentJob(S, file_lens, exps)
    job.upload(torch.from_numpy(host).pin_memory())
    job.run()
    rec, ifsc, fmd5, flags = job.download()
    m16 = job.md5_16k()
    torch.cuda.synchronize()
    assert flags.numpy().all()
    ifsc = ifsc.numpy().tobytes()
    fmd5 = fmd5.numpy().tobytes()
    desc = []
    for f, ln in enumerate(file_lens):
        n_sl = (ln + S - 1) // S
        desc.append({"name": names[f], "size": ln, "md5": fmd5[16 * f:16 * f + 16], "md5_16k": m16[f],
                     "ifsc": ifsc[20 * first[f]:20 * (first[f] + n_sl)]})
        assert m16[f] == hashlib.md5(files[f][:16384].tobytes()).digest()
    index, set_id, order = P.index_file(S, desc)

    # independent parse: every packet's length and MD5 check, set ID everywhere
    pk = list(P.parse(index))
    assert all(sid == set_id for _, sid, _ in pk)
    types = [t for t, _, _ in pk]
    assert types[0] == P.T_MAIN and types[-1] == P.T_CREATOR
    main_body = pk[0][2]
    assert hashlib.md5(main_body).digest() == set_id
    slice_size, nfiles = struct.unpack_from("<QI", main_body)
    assert (slice_size, nfiles) == (S, len(file_lens))
    ids = [main_body[12 + 16 * k:28 + 16 * k] for k in range(nfiles)]
    assert ids == order == P.sort_file_ids(ids)
    # FileDesc / IFSC contents against the oracle
    by_id = {}
    for t, _, body in pk:
        if t in (P.T_DESC, P.T_IFSC):
            by_id.setdefault(body[:16], {})[t] = body
    for f, ln in enumerate(file_lens):
        fid = P.file_id(hashlib.md5(files[f][:16384].tobytes()).digest(), ln, names[f])
        d = by_id[fid][P.T_DESC]
        assert d[16:32] == hashlib.md5(files[f].tobytes()).digest()
        assert struct.unpack_from("<Q", d, 48)[0] == ln
        assert d[56:56 + len(names[f].encode())] == names[f].encode()
        assert by_id[fid][P.T_IFSC][16:] == O.hash_file(files[f], S)[0]
    assert P.T_UNI in types  # the non-ASCII name gets a UniFileN packet

    # recovery packets: GPU packet MD5 == MD5 of header tail + slice
    md5s = job.recovery_packet_md5s(set_id)
    ref = O.recover(host, lens, np.arange(N), exps)
    vol = b""
    for r, e in enumerate(exps):
        data = rec.numpy()[r].tobytes()
        assert data == ref[r].tobytes()
        pkt = P.recovery_packet(set_id, e, data, md5s[r])
        assert md5s[r] == hashlib.md5(pkt[32:]).digest()
        vol += pkt
    for t, sid, body in P.parse(vol):
        assert t == P.T_RECV and sid == set_id
