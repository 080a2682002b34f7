"""Parsing of the serving trace (host only): records per server and per
reset segment, and the slow-request breakdown."""
from bioshell_gb300.serving import read_trace, slow_requests

TRACE = """# server
# B,slot,batch,kind,bucket,rows,nreq,hand_ms,launch_begin_ms,launch_end_ms,event_ms,finish_ms,dev_grows,host_grows,grow_ms
# R,id,kind,bucket,q,submit_ms,done_ms,batch,status
B,0,0,0,0,10,1,1.000,1.010,1.500,2.500,2.600,0,0,0.000
R,1,0,0,10,0.500,2.600,0,0
# reset
B,1,0,0,0,300,2,5.000,5.010,9.000,12.000,12.100,3,1,3.500
B,0,1,0,1,4,1,6.000,6.010,6.200,6.900,7.000,0,0,0.000
R,2,0,0,100,1.000,12.100,0,0
R,3,0,0,200,2.000,12.100,0,0
R,4,0,1,4,5.500,7.000,1,0
R,5,1,-1,50,3.000,40.000,2,0
# server
R,9,0,0,1,0.000,1.000,0,5
"""


def test_read_trace_and_slow_requests(tmp_path):
    p = tmp_path / "t.csv"
    p.write_text(TRACE)
    servers = read_trace(str(p))
    assert len(servers) == 2
    segs = servers[0]["segments"]
    assert len(segs) == 2 and len(segs[0]["requests"]) == 1 and len(segs[1]["batches"]) == 2
    b = segs[1]["batches"][0]
    assert b["rows"] == 300 and b["dev_grows"] == 3 and abs(b["grow_ms"] - 3.5) < 1e-12
    slow = slow_requests(segs[1], percentile=50.0)
    # the two requests of the 300-row batch; the clustering job is not a query
    assert [s["id"] for s in slow] == [2, 3]
    s = slow[0]
    assert abs(s["wait"] - 4.0) < 1e-9 and abs(s["launch"] - 3.99) < 1e-9
    assert abs(s["device"] - 3.0) < 1e-9 and abs(s["finish"] - 0.1) < 1e-9 and s["grows"] == 4
    assert slow_requests(servers[1]["segments"][0]) == []  # failed requests are left out
