"""The steer and job structures smoke() hands to mpgpu_pede_run: built from
the oracle driver's structures by field name, the device-only fields
(structure passes on the device, monitoring, preconditioner, monitor file)
keep their zero defaults.  No GPU call."""
import ctypes as C

import oracle_ref as orc


def test_steer_and_job_from_oracle_structs(mp):
    d = mp.generate(mp.gen_config("telescope", ntracks=200))
    st = orc.make_steer(metsol=1, matsto=1, mitera=1)
    job, keep = orc.make_job(d)
    gst = mp.Steer(**{f: getattr(st, f) for f, _ in mp.Steer._fields_ if hasattr(st, f)})
    gjob = mp.Job(**{f: getattr(job, f) for f, _ in mp.Job._fields_ if hasattr(job, f)})
    assert gst.metsol == 1 and gst.matsto == 1 and gst.mitera == 1
    assert gst.structDevice == 0 and gst.monitor == 0 and gst.mbandw == 0
    assert gjob.nrec == job.nrec and not gjob.monPath
    assert C.sizeof(gst) == C.sizeof(mp.Steer)
