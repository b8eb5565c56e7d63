complex (rejected)                                                      CUA1    
             3             1             1             1
cua                        1             1             1             0
(10I8)          (10I8)          (4E20.12)           
       1       2
       1
  1.000000000000E+00
