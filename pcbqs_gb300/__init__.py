"""pcbqs_gb300: a GB300-native (sm_103a) static-fill and solve backend for pcbqs.

  backend.factory      the `gb300` fill backend of pcbqs's `pcbqs.static_backends` entry-point group
  geometry             host preparation of a mesh and its upload to the device
  fill                 device-resident fill of the moments, L and P (torch tensors over the C ABI)
  board                meshed boards: terminals, via fans, ports and the MQS node merging
"""
__version__ = '0.1.0'
