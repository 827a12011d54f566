sep_tiny history
n1=4 o1=0.0 d1=0.004 label1="time (s)"
n2=7
Appended by a later program:
n2=3 o2=-25.0 d2=12.5 label2='offset'
n3=2 o3=100 d3=25 label3=y esize=4
data_format="xdr_float" in=sep_tiny.H@
